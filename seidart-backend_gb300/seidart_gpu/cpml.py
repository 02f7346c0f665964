"""C-PML coefficient grids in the representation the reference solvers read.

The reference reads ``kappa_cpml.dat``, ``alpha_cpml.dat``, ``acoef_cpml.dat``,
``bcoef_cpml.dat`` and their ``_half`` variants as full padded grids
(src/fortran/cpmlfdtd.f08:253-261): ONE (kappa, alpha, a, b) value per cell,
shared by every derivative direction at that cell (e.g. :332-335).  The
frontend that writes them is not part of the reference, so this module
generates them from the published convolutional-PML recursion of
Komatitsch & Martin (2007), credited by the reference at
legacy/cpmlfdtd_cbindings.f95:790-794:

    d(s)     = d0 * s**NP,              d0 = -(NP+1) * vmax * ln(R) / (2 L)
    kappa(s) = 1 + (kappa_max - 1) * s**NP
    alpha(s) = alpha_max * (1 - s),     alpha_max = pi * f0
    b        = exp(-(d/kappa + alpha) * dt)
    a        = d * (b - 1) / (kappa * (d + kappa * alpha))   (0 where d ~ 0)

with s in [0, 1] the normalised depth into a PML of thickness L = cpml * h.
Each axis gets the 1D profile of the standard derivation (full-grid points
x = i h, half-grid points x = (i + 1/2) h); a cell's combined depth is the
largest of its per-axis depths (the corner regions take the deeper axis).
Outside the PML kappa = 1 and alpha = a = 0, b = 1, so the memory variables
stay exactly zero there.
"""
from __future__ import annotations

import numpy as np

NP = 2.0
R_COEF = 1.0e-3


def _depth_1d(n: int, cpml: int, half: bool) -> np.ndarray:
    """Normalised PML depth per grid index along one axis (-1 = not in the PML)."""
    h = 1.0
    L = cpml * h
    x = np.arange(n, dtype=np.float64) * h + (0.5 * h if half else 0.0)
    left = L - x
    right = x - ((n - 1) * h - L)
    depth = np.full(n, -1.0)
    m = left >= 0
    depth[m] = left[m] / L
    m = right >= 0
    depth[m] = np.maximum(depth[m], right[m] / L)
    return np.minimum(depth, 1.0)


def cpml_grids(shape, cpml: int, spacing, dt: float, vmax: float, f0: float,
               kappa_max: float = 2.0) -> dict:
    """Return the eight CPML grids for a padded grid of ``shape`` (x fastest,
    Fortran order) as a dict with keys kappa, alpha, acoef, bcoef and the
    ``_half`` variants."""
    shape = tuple(int(s) for s in shape)
    if cpml <= 0:
        ones, zeros = np.ones(shape, order="F"), np.zeros(shape, order="F")
        return {"kappa": ones, "alpha": zeros, "acoef": zeros, "bcoef": ones,
                "kappa_half": ones.copy(), "alpha_half": zeros.copy(), "acoef_half": zeros.copy(),
                "bcoef_half": ones.copy()}
    alpha_max = np.pi * f0
    out = {}
    for half in (False, True):
        depth = None
        d0_axis = []
        for ax, n in enumerate(shape):
            L = cpml * float(spacing[ax])
            d0_axis.append(-(NP + 1.0) * vmax * np.log(R_COEF) / (2.0 * L))
            dd = _depth_1d(n, cpml, half)
            view = [1] * len(shape)
            view[ax] = n
            dd = dd.reshape(view)
            depth = dd if depth is None else np.maximum(depth, dd)
        depth = np.broadcast_to(depth, shape)
        inside = depth >= 0.0
        s = np.where(inside, depth, 0.0)
        d0 = max(d0_axis)
        d = np.where(inside, d0 * s ** NP, 0.0)
        kappa = np.where(inside, 1.0 + (kappa_max - 1.0) * s ** NP, 1.0)
        alpha = np.where(inside, alpha_max * (1.0 - s), 0.0)
        alpha = np.maximum(alpha, 0.0)
        b = np.exp(-(d / kappa + alpha) * dt)
        with np.errstate(divide="ignore", invalid="ignore"):
            a = np.where(np.abs(d) > 1.0e-6, d * (b - 1.0) / (kappa * (d + kappa * alpha)), 0.0)
        sfx = "_half" if half else ""
        for name, arr in (("kappa", kappa), ("alpha", alpha), ("acoef", a), ("bcoef", b)):
            out[name + sfx] = np.asfortranarray(arr.astype(np.float64))
    return out
