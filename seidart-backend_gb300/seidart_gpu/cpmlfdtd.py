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

__all__ = ["seismic2", "seismic25", "electromag2", "electromag25", "electromag2c", "electromag25c",
           "permittivity_write", "permittivity_write_c", "stiffness_write", "attenuation_write"]

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


# ---------------------------------------------------------- material writers
# The binding's writers take (im, mlist, npoints_pml, nx, nz)
# (legacy/cpmlfdtd_wrapper.c:19-137) and write the padded .dat records into
# the working directory.  Fortran reads im(nx, nz) from the array's memory,
# x fastest, so the image is taken the same way here; the table is the
# (nmat, ncol) array.  The binding's prototypes drop stiffness_write's
# gradient and attenuation_write's cpmlvalue; both are keyword arguments here.
def _image(im, nx, nz):
    a = np.ascontiguousarray(im, dtype=np.int32).reshape(-1)
    if a.size != nx * nz:
        raise ValueError(f"im holds {a.size} cells, expected nx * nz = {nx * nz}")
    return a.reshape((nx, nz), order="F")


def permittivity_write(im, mlist, npoints_pml, nx, nz):
    from . import material
    material.permittivity_write(".", _image(im, nx, nz), np.asarray(mlist, dtype=np.float64), int(npoints_pml))


def permittivity_write_c(im, mlist, npoints_pml, nx, nz):
    from . import material
    material.permittivity_write(".", _image(im, nx, nz), np.asarray(mlist, dtype=np.complex128), int(npoints_pml),
                                complex_valued=True)


def stiffness_write(im, mlist, npoints_pml, nx, nz, gradient=None):
    from . import material
    g = None if gradient is None else np.asarray(gradient, dtype=np.float64).reshape((nx, nz), order="F")
    material.stiffness_write(".", _image(im, nx, nz), np.asarray(mlist, dtype=np.float64), int(npoints_pml), g)


def attenuation_write(im, alist, npoints_pml, nx, nz, cpmlvalue=0.0):
    from . import material
    material.attenuation_write(".", _image(im, nx, nz), np.asarray(alist, dtype=np.float64), int(npoints_pml),
                               float(cpmlvalue))
