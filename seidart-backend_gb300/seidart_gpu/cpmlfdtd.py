"""Drop-in module with the reference's Python entry points.

Mirrors ``seidart.fortran.cpmlfdtd`` (legacy/__init__.py:2-12,
legacy/cpmlfdtd_wrapper.py:13-43, legacy/cpmlfdtd_wrapper.c:139-375): the
solver functions take the argument layout of the CPython wrapper
``(nx, nz, dx, dz, src, npoints_pml, nstep[, single_output])`` (seismic25,
electromag25[c]: ``(nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep[,
single_output])``), read the .dat inputs from the working directory and
write the per-step snapshot files there, like the reference.  The binding's
seismic25 and electromag25 are 3D solvers with 3D snapshots
(legacy/cpmlfdtd_cbindings.f95:1088, :2184); they run the 3D loops
(seismic3, electromag3).  Each call goes through ctypes to the C entry
points seismic2_ ... electromag25c_ of libseidart_gpu.so.

nx, nz (ny) are the padded grid sizes; ``src`` holds the interior source
indices (x, z) or (x, y, z).  Errors raise SeidartError (the reference's
binding returns None and stops the process on failure).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SeidartError, lib

__all__ = ["seismic2", "seismic25", "electromag2", "electromag25", "electromag2c", "electromag25c"]

_DECL = False


def _declare():
    global _DECL
    if _DECL:
        return
    L = lib()
    two = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_int, C.c_int]
    three = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_int, C.c_int]
    for name, args in (("seismic2_", two), ("electromag2_", two), ("electromag2c_", two),
                       ("seismic25_", three), ("electromag25_", three), ("electromag25c_", three)):
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = None
    L.seidart_io_last_error.restype = C.c_char_p
    _DECL = True


def _src(src, n):
    a = np.ascontiguousarray(np.asarray(src, dtype=np.int32).ravel())
    if a.size < n:
        raise ValueError(f"src needs {n} source indices")
    return a


def _call2(name, nx, nz, dx, dz, src, npoints_pml, nstep, single_output):
    _declare()
    L = lib()
    L.seidart_io_last_error  # ensure declared
    s = _src(src, 2)
    before = L.seidart_io_last_error()
    getattr(L, name)(int(nx), int(nz), float(dx), float(dz), int(npoints_pml), s.ctypes.data, int(nstep),
                     1 if single_output else 0)
    after = L.seidart_io_last_error()
    if after and after != before:
        raise SeidartError(-4, after.decode(errors="replace"))


def _call3(name, nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep, single_output):
    _declare()
    L = lib()
    s = _src(src, 3)
    before = L.seidart_io_last_error()
    getattr(L, name)(int(nx), int(ny), int(nz), float(dx), float(dy), float(dz), int(npoints_pml), s.ctypes.data,
                     int(nstep), 1 if single_output else 0)
    after = L.seidart_io_last_error()
    if after and after != before:
        raise SeidartError(-4, after.decode(errors="replace"))


def seismic2(nx, nz, dx, dz, src, npoints_pml, nstep, single_output=True):
    _call2("seismic2_", nx, nz, dx, dz, src, npoints_pml, nstep, single_output)


def electromag2(nx, nz, dx, dz, src, npoints_pml, nstep, single_output=True):
    _call2("electromag2_", nx, nz, dx, dz, src, npoints_pml, nstep, single_output)


def electromag2c(nx, nz, dx, dz, src, npoints_pml, nstep, single_output=True):
    _call2("electromag2c_", nx, nz, dx, dz, src, npoints_pml, nstep, single_output)


def seismic25(nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep, single_output=True):
    _call3("seismic25_", nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep, single_output)


def electromag25(nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep, single_output=True):
    _call3("electromag25_", nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep, single_output)


def electromag25c(nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep, single_output=True):
    _call3("electromag25c_", nx, ny, nz, dx, dy, dz, src, npoints_pml, nstep, single_output)
