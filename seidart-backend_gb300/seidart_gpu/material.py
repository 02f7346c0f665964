"""Material pre-pass: a material-ID image expanded into the padded coefficient
grids the solvers read (the reference's stiffness_write, attenuation_write
and permittivity_write[_c], legacy/cpmlfdtd_cbindings.f95:60-611), either
returned as arrays or written as the reference's ``.dat`` records.

``im`` is an (nx, nz) integer image of 1-based rows of the material table
(the reference reads ``mlist(im(i, j), col)``); tables are (nmat, ncol)
arrays in the reference's column convention (see include/seidart_gpu.h).
Outputs are (nx + 2 npml, nz + 2 npml) FP64 grids in Fortran order.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ._lib import SeidartError, lib, ptr_array

STIFFNESS_NAMES = ["c11", "c12", "c13", "c14", "c15", "c16", "c22", "c23", "c24", "c25", "c26",
                   "c33", "c34", "c35", "c36", "c44", "c45", "c46", "c55", "c56", "c66", "rho"]
EPS_NAMES = ["eps11", "eps12", "eps13", "eps22", "eps23", "eps33"]
SIG_NAMES = ["sig11", "sig12", "sig13", "sig22", "sig23", "sig33"]
GAMMA_NAMES = ["gamma_x", "gamma_y", "gamma_z"]

_DECL = False


def _declare():
    global _DECL
    if _DECL:
        return
    L = lib()
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    sig = {
        "seidart_stiffness_arrays": [vp, i, i, vp, i, i, i, vp, vp],
        "seidart_stiffness_write": [C.c_char_p, vp, i, i, vp, i, i, i, vp],
        "seidart_permittivity_arrays": [vp, i, i, vp, i, i, i, vp],
        "seidart_permittivity_write": [C.c_char_p, vp, i, i, vp, i, i, i],
        "seidart_permittivity_arrays_c": [vp, i, i, vp, i, i, i, vp],
        "seidart_permittivity_write_c": [C.c_char_p, vp, i, i, vp, i, i, i],
        "seidart_attenuation_arrays": [vp, i, i, vp, i, i, i, d, vp],
        "seidart_attenuation_write": [C.c_char_p, vp, i, i, vp, i, i, i, d],
        "seidart_stiffness_arrays_dev": [vp, i, i, vp, i, i, i, vp, vp, vp],
        "seidart_permittivity_arrays_dev": [vp, i, i, vp, i, i, i, vp, vp],
        "seidart_permittivity_arrays_c_dev": [vp, i, i, vp, i, i, i, vp, vp],
        "seidart_attenuation_arrays_dev": [vp, i, i, vp, i, i, i, d, vp, vp],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = C.c_int, args
    _DECL = True


def _check(rc: int) -> None:
    if rc != 0:
        raise SeidartError(rc, lib().seidart_last_error().decode(errors="replace"))


def _inputs(im, table, dtype=np.float64):
    _declare()
    im = np.asfortranarray(im, dtype=np.int32)
    if im.ndim != 2:
        raise ValueError("im must be an (nx, nz) image")
    table = np.ascontiguousarray(table, dtype=dtype)
    if table.ndim != 2:
        raise ValueError("the material table must be (nmat, ncol)")
    return im, table


def _grids(n, shape, dtype=np.float64):
    return [np.zeros(shape, dtype=dtype, order="F") for _ in range(n)]


def stiffness_arrays(im, mlist, npml: int, gradient=None) -> dict:
    """{c11 .. c66, rho} padded grids (gradient scales the interior density)."""
    im, mlist = _inputs(im, mlist)
    nx, nz = im.shape
    shape = (nx + 2 * npml, nz + 2 * npml)
    out = _grids(22, shape)
    g = None if gradient is None else np.asfortranarray(gradient, dtype=np.float64)
    _check(lib().seidart_stiffness_arrays(im.ctypes.data, nx, nz, mlist.ctypes.data, mlist.shape[0], mlist.shape[1],
                                          int(npml), None if g is None else g.ctypes.data, ptr_array(out)))
    return dict(zip(STIFFNESS_NAMES, out))


def permittivity_arrays(im, mlist, npml: int, complex_valued: bool = False) -> dict:
    """{eps11 .. eps33, sig11 .. sig33} padded grids; with ``complex_valued``
    the table is complex, eps grids are complex and sig = |table value|."""
    im, mlist = _inputs(im, mlist, np.complex128 if complex_valued else np.float64)
    nx, nz = im.shape
    shape = (nx + 2 * npml, nz + 2 * npml)
    eps = _grids(6, shape, np.complex128 if complex_valued else np.float64)
    sig = _grids(6, shape)
    fn = lib().seidart_permittivity_arrays_c if complex_valued else lib().seidart_permittivity_arrays
    _check(fn(im.ctypes.data, nx, nz, mlist.ctypes.data, mlist.shape[0], mlist.shape[1], int(npml),
              ptr_array(eps + sig)))
    return dict(zip(EPS_NAMES + SIG_NAMES, eps + sig))


def attenuation_arrays(im, alist, npml: int, cpmlvalue: float) -> dict:
    """{gamma_x, gamma_y, gamma_z} padded grids; the CPML holds ``cpmlvalue``."""
    im, alist = _inputs(im, alist)
    nx, nz = im.shape
    out = _grids(3, (nx + 2 * npml, nz + 2 * npml))
    _check(lib().seidart_attenuation_arrays(im.ctypes.data, nx, nz, alist.ctypes.data, alist.shape[0],
                                            alist.shape[1], int(npml), float(cpmlvalue), ptr_array(out)))
    return dict(zip(GAMMA_NAMES, out))


def stiffness_write(directory, im, mlist, npml: int, gradient=None) -> None:
    """c11.dat .. c66.dat, rho.dat in ``directory`` (the reference's stiffness_write)."""
    im, mlist = _inputs(im, mlist)
    g = None if gradient is None else np.asfortranarray(gradient, dtype=np.float64)
    _check(lib().seidart_stiffness_write(str(Path(directory)).encode(), im.ctypes.data, im.shape[0], im.shape[1],
                                         mlist.ctypes.data, mlist.shape[0], mlist.shape[1], int(npml),
                                         None if g is None else g.ctypes.data))


def permittivity_write(directory, im, mlist, npml: int, complex_valued: bool = False) -> None:
    """eps11.dat .. sig33.dat in ``directory`` (permittivity_write[_c])."""
    im, mlist = _inputs(im, mlist, np.complex128 if complex_valued else np.float64)
    fn = lib().seidart_permittivity_write_c if complex_valued else lib().seidart_permittivity_write
    _check(fn(str(Path(directory)).encode(), im.ctypes.data, im.shape[0], im.shape[1], mlist.ctypes.data,
              mlist.shape[0], mlist.shape[1], int(npml)))


def attenuation_write(directory, im, alist, npml: int, cpmlvalue: float) -> None:
    """gamma_x.dat, gamma_y.dat, gamma_z.dat in ``directory`` (attenuation_write)."""
    im, alist = _inputs(im, alist)
    _check(lib().seidart_attenuation_write(str(Path(directory)).encode(), im.ctypes.data, im.shape[0], im.shape[1],
                                           alist.ctypes.data, alist.shape[0], alist.shape[1], int(npml),
                                           float(cpmlvalue)))


# ------------------------------------------------------------ on the device
def _device_grids(n, nx, nz, npml, complex_valued=False):
    import torch
    dt = torch.complex128 if complex_valued else torch.float64
    # row-major (NZ, NX) is the Fortran (NX, NZ) layout the solvers read
    return [torch.empty((nz + 2 * npml, nx + 2 * npml), dtype=dt, device="cuda") for _ in range(n)]


def _stream_ptr(stream):
    import torch
    return (stream or torch.cuda.current_stream()).cuda_stream


def stiffness_arrays_device(im, mlist, npml: int, gradient=None, stream=None) -> dict:
    """The stiffness pre-pass run on the device: {c11 .. c66, rho} as CUDA
    FP64 tensors of shape (nz + 2 npml, nx + 2 npml) -- row-major, so the
    memory is the Fortran (nx, nz) grid the solvers read; ``fortran(t)``
    gives the NumPy view.  Bit-identical to :func:`stiffness_arrays`."""
    im, mlist = _inputs(im, mlist)
    nx, nz = im.shape
    out = _device_grids(22, nx, nz, npml)
    g = None if gradient is None else np.asfortranarray(gradient, dtype=np.float64)
    ptrs = (C.c_void_p * 22)(*[t.data_ptr() for t in out])
    _check(lib().seidart_stiffness_arrays_dev(im.ctypes.data, nx, nz, mlist.ctypes.data, mlist.shape[0],
                                              mlist.shape[1], int(npml), None if g is None else g.ctypes.data, ptrs,
                                              _stream_ptr(stream)))
    return dict(zip(STIFFNESS_NAMES, out))


def permittivity_arrays_device(im, mlist, npml: int, complex_valued: bool = False, stream=None) -> dict:
    """The permittivity pre-pass on the device (see stiffness_arrays_device)."""
    im, mlist = _inputs(im, mlist, np.complex128 if complex_valued else np.float64)
    nx, nz = im.shape
    eps = _device_grids(6, nx, nz, npml, complex_valued)
    sig = _device_grids(6, nx, nz, npml)
    ptrs = (C.c_void_p * 12)(*[t.data_ptr() for t in eps + sig])
    fn = lib().seidart_permittivity_arrays_c_dev if complex_valued else lib().seidart_permittivity_arrays_dev
    _check(fn(im.ctypes.data, nx, nz, mlist.ctypes.data, mlist.shape[0], mlist.shape[1], int(npml), ptrs,
              _stream_ptr(stream)))
    return dict(zip(EPS_NAMES + SIG_NAMES, eps + sig))


def attenuation_arrays_device(im, alist, npml: int, cpmlvalue: float, stream=None) -> dict:
    """The attenuation pre-pass on the device (see stiffness_arrays_device)."""
    im, alist = _inputs(im, alist)
    nx, nz = im.shape
    out = _device_grids(3, nx, nz, npml)
    ptrs = (C.c_void_p * 3)(*[t.data_ptr() for t in out])
    _check(lib().seidart_attenuation_arrays_dev(im.ctypes.data, nx, nz, alist.ctypes.data, alist.shape[0],
                                                alist.shape[1], int(npml), float(cpmlvalue), ptrs,
                                                _stream_ptr(stream)))
    return dict(zip(GAMMA_NAMES, out))


def fortran(t) -> np.ndarray:
    """A device grid of the *_device functions as a host (nx, nz) array in
    Fortran order."""
    return t.cpu().numpy().T
