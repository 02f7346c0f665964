"""The C-ABI library loads without a GPU and exports every function that
include/seidart_gpu.h declares (no compute calls here)."""
import ctypes
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

HEADER = ROOT / "include" / "seidart_gpu.h"


def _declared() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"^\s*#[^\n]*", "", text, flags=re.M)
    names = set()
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
        name = m.group(1)
        before = text[:m.start()].rstrip()
        # a declaration: the name follows a return type, not an operator or '('
        if before and (before[-1].isalnum() or before[-1] in "*_") and not before.endswith(("sizeof", "return")):
            names.add(name)
    return sorted(names)


def _lib():
    from seidart_gpu import _lib as L
    if not L.LIB_PATH.exists():
        pytest.skip("libseidart_gpu.so is not built")
    return ctypes.CDLL(str(L.LIB_PATH))


def test_header_declares_the_entry_points():
    names = _declared()
    for n in ("seidart_solver_create", "seidart_run", "seidart_run_files", "seismic2_", "electromag25c_",
              "seidart_batch_create", "seidart_fwi_gradient", "seidart_trace_misfit_noalloc", "seidart_cli_main"):
        assert n in names


def test_library_exports_every_declared_function():
    lib = _lib()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_unresolved_internal_symbols():
    from seidart_gpu import _lib as L
    if not L.LIB_PATH.exists() or not shutil.which("nm"):
        pytest.skip("library or nm missing")
    out = subprocess.run(["nm", "-D", "--undefined-only", str(L.LIB_PATH)], capture_output=True, text=True).stdout
    # every undefined symbol must come from a versioned system library (libc, libstdc++, libgcc, libm)
    unversioned = [ln.split()[-1] for ln in out.splitlines() if ln.strip() and "@" not in ln]
    unversioned = [s for s in unversioned if not s.startswith(("__gmon_start__", "_ITM_", "__cxa_finalize"))]
    assert not unversioned, unversioned


def test_python_constants_match_the_header():
    """Family and precision codes of the Python package are the header's."""
    import seidart_gpu as sg
    text = HEADER.read_text()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(SEIDART_[A-Z0-9_]+)\s+(-?\d+)", text)}
    for name in ("FP64", "FP32", "FP64_FAST", "SEISMIC2", "SEISMIC25", "SEISMIC3", "ELECTROMAG2", "ELECTROMAG25",
                 "ELECTROMAG3"):
        assert defs["SEIDART_" + name] == getattr(sg, name), name
