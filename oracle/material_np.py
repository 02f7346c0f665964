"""NumPy restatement of the material pre-pass -- TEST INFRASTRUCTURE.

Only tests import this module.  It follows the statements of
legacy/cpmlfdtd_cbindings.f95 one by one (0-based here: Fortran index i is
Python index i-1): permittivity_write (:60-201), permittivity_write_c
(:204-348, sigma = |table value|), stiffness_write (:351-562) and
attenuation_write (:565-611).  Each array assignment evaluates its right
side before writing, as Fortran array assignment does.
"""
from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np

# |z| as the reference's abs(complex) gets it: the C library's cabs/hypot
# (gfortran calls cabs); NumPy's vectorised array path rounds differently
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.hypot.restype = ctypes.c_double
_libm.hypot.argtypes = [ctypes.c_double, ctypes.c_double]


def _cabs(a):
    out = np.empty(a.shape, dtype=np.float64)
    flat, src = out.reshape(-1), a.reshape(-1)
    for q in range(src.size):
        flat[q] = _libm.hypot(src[q].real, src[q].imag)
    return out


def _fill(im, table, P, col0, count, dtype=np.float64):
    nx, nz = im.shape
    out = []
    for a in range(count):
        g = np.zeros((nx + 2 * P, nz + 2 * P), dtype=dtype)
        g[P:P + nx, P:P + nz] = table[im - 1, col0 - 1 + a]
        out.append(g)
    return out


def stiffness(im, mlist, P, gradient=None):
    nx, nz = im.shape
    g = _fill(im, mlist, P, 2, 22)
    if gradient is not None:
        g[21][P:P + nx, P:P + nz] = g[21][P:P + nx, P:P + nz] * gradient
    for i in range(1, P + 2):
        for a in g:                                   # top
            a[i - 1, :] = a[P, :].copy()
        for a in g:                                   # bottom
            a[nx + P - 1 + i - 1, :] = a[nx + P - 2, :].copy()
        for a in g:                                   # left
            a[:, i - 1] = a[:, P].copy()
        for a in g:                                   # right
            a[:, nz + P - 1 + i - 1] = a[:, nz + P - 2].copy()
    return g


def permittivity(im, mlist, P, complex_valued=False):
    nx, nz = im.shape
    if complex_valued:
        eps = _fill(im, mlist, P, 2, 6, np.complex128)
        sig = [_cabs(x) for x in _fill(im, mlist, P, 8, 6, np.complex128)]
    else:
        eps = _fill(im, mlist, P, 2, 6)
        sig = _fill(im, mlist, P, 8, 6)
    e11, e12, e13, e22, e23, e33 = eps
    s11, s12, s13, s22, s23, s33 = sig
    ref_order_e = [e11, e22, e33, e12, e13, e23]
    hx, sx = nx + P - 1, nx + P - 2       # 0-based: row nx+P-1+i and row nx+P-1
    hz, sz = nz + P - 1, nz + P - 2
    for i in range(1, P + 2):
        for a in ref_order_e:
            a[i - 1, :] = a[P, :].copy()
        for a in ref_order_e:
            a[hx + i - 1, :] = a[sx, :].copy()
        for a in (s11, s22, s33, s12, s13, s23):
            a[i - 1, :] = a[P, :].copy()
        s11[hx + i - 1, :] = s11[sx, :].copy()
        s22[hx + i - 1, :] = s22[sx, :].copy()
        s33[hx + i - 1, :] = s33[sx, :].copy()
        s13[hx + i - 1, :] = s12[sx, :].copy()
        s13[hx + i - 1, :] = s13[sx, :].copy()
        s23[hx + i - 1, :] = s23[sx, :].copy()
        for a in ref_order_e:
            a[:, i - 1] = a[:, P].copy()
        for a in ref_order_e:
            a[:, hz + i - 1] = a[:, sz].copy()
        s11[:, i - 1] = s11[:, P].copy()
        s22[:, i - 1] = s22[:, P].copy()
        s33[:, i - 1] = s33[:, P].copy()
        s12[:, i - 1] = s11[:, P].copy()
        s13[:, i - 1] = s13[:, P].copy()
        s23[:, i - 1] = s33[:, P].copy()
        for a in (s11, s22, s33, s12, s13, s23):
            a[:, hz + i - 1] = a[:, sz].copy()
    return eps + sig


def attenuation(im, alist, P, cpmlvalue):
    nx, nz = im.shape
    out = []
    for a in range(3):
        g = np.full((nx + 2 * P, nz + 2 * P), cpmlvalue, dtype=np.float64)
        g[P:P + nx, P:P + nz] = alist[im - 1, a]
        out.append(g)
    return out
