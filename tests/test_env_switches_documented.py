"""Every environment variable the native library reads is listed in the
user-facing integration notes, so a switch cannot be added silently."""
import pathlib
import re

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_every_getenv_is_documented():
    names = set()
    for src in (ROOT / "seidart-backend_gb300" / "csrc").glob("*.c*"):
        names |= set(re.findall(r'getenv\("(SEIDART_[A-Z0-9_]+)"\)', src.read_text()))
    for src in (ROOT / "seidart-backend_gb300" / "csrc").glob("*.h"):
        names |= set(re.findall(r'getenv\("(SEIDART_[A-Z0-9_]+)"\)', src.read_text()))
    assert names, "no environment switches found"
    doc = (ROOT / "INTEGRATION.md").read_text()
    missing = sorted(n for n in names if n not in doc)
    assert not missing, f"undocumented environment switches: {missing}"
