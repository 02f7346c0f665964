"""zstd frames of the 2.5D block output (seidart_zstd_write, host code: runs
without a GPU).  The library path (system libzstd, level 3) and the raw-block
fallback both decode to the input bytes, for empty data, one short block
and several 128 KiB blocks."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from seidart_gpu import _lib
from seidart_gpu.fortran_io import _raw_frame, _zstd_lib, read_zstd

pytestmark = pytest.mark.skipif(not _lib.LIB_PATH.exists(), reason="library not built")

SIZES = [0, 12, 128 * 1024, 3 * 128 * 1024 + 4]


def _write(path, data: bytes):
    L = C.CDLL(str(_lib.LIB_PATH))
    L.seidart_zstd_write.restype = C.c_int
    L.seidart_zstd_write.argtypes = [C.c_char_p, C.c_void_p, C.c_size_t]
    buf = C.create_string_buffer(data, max(len(data), 1))
    assert L.seidart_zstd_write(str(path).encode(), buf, len(data)) == 0


@pytest.mark.parametrize("n", SIZES)
def test_frame_round_trip(tmp_path, n):
    data = np.random.default_rng(n).standard_normal(n // 4 + 1).astype(np.float32).tobytes()[:n]
    p = tmp_path / "a.zst"
    _write(p, data)
    assert read_zstd(p) == data
    if _zstd_lib() is not None and n >= 128 * 1024:
        assert p.stat().st_size < n  # compressed by libzstd


def test_raw_fallback_frames(tmp_path):
    """SEIDART_ZSTD_RAW=1 writes raw blocks; both the raw parser and libzstd
    (when present) read them."""
    code = (
        "import sys, numpy as np, ctypes as C\n"
        "from seidart_gpu import _lib\n"
        "L = C.CDLL(str(_lib.LIB_PATH))\n"
        "L.seidart_zstd_write.argtypes = [C.c_char_p, C.c_void_p, C.c_size_t]\n"
        "for n in %r:\n"
        "    d = np.arange(n, dtype=np.uint8).tobytes()\n"
        "    b = C.create_string_buffer(d, max(n, 1))\n"
        "    assert L.seidart_zstd_write(('%s/r%%d.zst' %% n).encode(), b, n) == 0\n" % (SIZES, tmp_path))
    env = {**os.environ, "SEIDART_ZSTD_RAW": "1"}
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env["PYTHONPATH"] = os.pathsep.join([os.path.join(root, "seidart-backend_gb300"), root])
    subprocess.run([sys.executable, "-c", code], check=True, env=env)
    for n in SIZES:
        buf = (tmp_path / f"r{n}.zst").read_bytes()
        want = np.arange(n, dtype=np.uint8).tobytes()
        assert len(buf) == n + 14 + 3 * max(1, -(-n // (128 * 1024)))
        assert _raw_frame(buf) == want
        if _zstd_lib() is not None:
            assert read_zstd(tmp_path / f"r{n}.zst") == want
