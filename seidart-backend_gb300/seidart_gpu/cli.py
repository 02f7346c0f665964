"""``python -m seidart_gpu.cli <input.json> [seismic=true|false] [density_method=...]``

Same behaviour as the reference's ``seidartfdtd`` executable
(src/fortran/main.f08): parses input.json, pads the grid by 2*cpml, reads the
.dat inputs from the working directory, runs the GPU solver and writes the
per-step snapshot files.  The compiled ``seidartfdtd`` binary next to this
file is the same driver without Python.
"""
from __future__ import annotations

import ctypes as C
import sys

from ._lib import lib


def main(argv=None) -> int:
    argv = list(sys.argv if argv is None else argv)
    L = lib()
    L.seidart_cli_main.restype = C.c_int
    L.seidart_cli_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
    sys.stdout.flush()
    return int(L.seidart_cli_main(len(argv), arr))


if __name__ == "__main__":
    sys.exit(main(["seidartfdtd", *sys.argv[1:]]))
