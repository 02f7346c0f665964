"""Known-answer cases for the CPML-FDTD solvers, built from analytic values
rather than from the CPU restatement.

Manufactured fields.  The reference's stress loops use the staggered
fourth-order difference (27 (f(x+h/2) - f(x-h/2)) - (f(x+3h/2) - f(x-3h/2))) /
(24 h), which is exact for polynomials up to degree 4, so one stress
half-step applied to polynomial velocities gives the analytic strain rates at
the staggered points (src/fortran/cpmlfdtd.f08:324-386 in 2D, :1761-1992 in
3D).  Its velocity loops use three-term forms instead
(cpmlfdtd.f08:405-406, :434-435, :2022-2024, :2063-2066, :2107-2111):

  "backward"  (27 s(i) - 27 s(i-1) + s(i-2)) / (24 h)
              = exact derivative at i - 1/2 + s(i+1) / (24 h)
  "forward"   (-27 s(i) + 27 s(i+1) - s(i+2)) / (24 h)
              = exact derivative at i + 1/2 - s(i-1) / (24 h)

for stresses of degree <= 4 (here they are quadratic), so one whole time
step from polynomial velocities and zero stresses has a closed form: the
analytic derivative plus the extra term each three-term form carries.  The
extra term is a zeroth-order term (the forms are not consistent
approximations of a derivative); the drop-in reproduces it because the
reference computes it.

Only cells of the inert interior (kappa = 1, a = 0, no attenuation), at
least three cells from its faces, are checked, so no CPML memory or
boundary ring enters.
"""
from __future__ import annotations

import dataclasses

import numpy as np
from numpy.polynomial import polynomial as P

from seidart_gpu import models
from seidart_gpu.api import C21, Problem

# ------------------------------------------------------------------ 2D
ANISO2 = dict(c11=9.0e9, c13=4.0e9, c15=0.6e9, c33=11.0e9, c35=-0.4e9, c55=2.5e9)


def _poly2(rng, deg: int = 3) -> np.ndarray:
    c = np.zeros((deg + 1, deg + 1))
    for a in range(deg + 1):
        for b in range(deg + 1 - a):
            c[a, b] = rng.uniform(-1.0, 1.0)
    return c


def seismic2_manufactured(n: int = 40, cpml: int = 8, dt: float = 1e-3, rho: float = 1800.0, seed: int = 11):
    """A homogeneous anisotropic seismic2 problem with cubic initial
    velocities (unit-scaled coordinates x/n, z/n), one time step, zero
    sources.  Returns (problem, expected) where expected maps field name ->
    (values, mask) of the closed-form state after the step."""
    rng = np.random.default_rng(seed)
    nx = nz = n + 2 * cpml
    h = 1.0
    L = float(n)
    cx, cz = _poly2(rng), _poly2(rng)   # vx, vz in unit coordinates

    def ev(c, x, z, dx=0, dz=0):
        cc = c
        if dx:
            cc = P.polyder(cc, dx, axis=0)
        if dz:
            cc = P.polyder(cc, dz, axis=1)
        return P.polyval2d(x / L, z / L, cc) / L ** (dx + dz)

    i = np.arange(nx, dtype=np.float64)[:, None]
    j = np.arange(nz, dtype=np.float64)[None, :]
    X, Z = i * h + 0 * j, 0 * i + j * h
    vx0 = np.asfortranarray(ev(cx, X, Z))
    vz0 = np.asfortranarray(ev(cz, X, Z))
    c = ANISO2
    # normal-stress loop (:324-353): forward x, backward z
    dvx_dx, dvz_dz = ev(cx, X + 0.5, Z, dx=1), ev(cz, X, Z - 0.5, dz=1)
    dvz_dx, dvx_dz = ev(cz, X + 0.5, Z, dx=1), ev(cx, X, Z - 0.5, dz=1)
    sxx = dt * (c["c11"] * dvx_dx + c["c13"] * dvz_dz + c["c15"] * (dvz_dx + dvx_dz))
    szz = dt * (c["c13"] * dvx_dx + c["c33"] * dvz_dz + c["c35"] * (dvz_dx + dvx_dz))
    # shear loop (:362-386): backward x, forward z
    dvx_dx, dvz_dz = ev(cx, X - 0.5, Z, dx=1), ev(cz, X, Z + 0.5, dz=1)
    dvz_dx, dvx_dz = ev(cz, X - 0.5, Z, dx=1), ev(cx, X, Z + 0.5, dz=1)
    sxz = dt * (c["c15"] * dvx_dx + c["c35"] * dvz_dz + c["c55"] * (dvz_dx + dvx_dz))

    # the stresses are quadratics in (x, z); their exact derivatives at the
    # half points come from the same closed forms, differentiated once more
    def s_poly(kind):
        """coefficients (in unit coordinates) of sxx, szz or sxz as polynomials"""
        if kind == "sxz":
            sh = [(-0.5, 0.0), (0.0, 0.5), (-0.5, 0.0), (0.0, 0.5)]
            w = [c["c15"], c["c35"], c["c55"], c["c55"]]
        else:
            sh = [(0.5, 0.0), (0.0, -0.5), (0.5, 0.0), (0.0, -0.5)]
            w = ([c["c11"], c["c13"], c["c15"], c["c15"]] if kind == "sxx" else
                 [c["c13"], c["c33"], c["c35"], c["c35"]])
        terms = [(cx, 1, 0), (cz, 0, 1), (cz, 1, 0), (cx, 0, 1)]
        tot = np.zeros((4, 4))
        for (coef, ddx, ddz), (shx, shz), ww in zip(terms, sh, w):
            d = P.polyder(coef, ddx, axis=0) if ddx else P.polyder(coef, ddz, axis=1)
            d = d / L
            shifted = _shift2(d, shx / L, shz / L)
            tot[:shifted.shape[0], :shifted.shape[1]] += ww * shifted
        return dt * tot

    psxx, pszz, psxz = s_poly("sxx"), s_poly("szz"), s_poly("sxz")

    def sv(pc, x, z, dx=0, dz=0):
        cc = pc
        if dx:
            cc = P.polyder(cc, dx, axis=0)
        if dz:
            cc = P.polyder(cc, dz, axis=1)
        return P.polyval2d(x / L, z / L, cc) / L ** (dx + dz)

    # vx (:399-416): backward three-term forms in x and z
    vx1 = vx0 + dt / rho * (sv(psxx, X - 0.5, Z, dx=1) + sv(psxx, X + 1, Z) / (24 * h)
                            + sv(psxz, X, Z - 0.5, dz=1) + sv(psxz, X, Z + 1) / (24 * h))
    # vz (:428-446): forward three-term forms in x and z
    vz1 = vz0 + dt / rho * (sv(psxz, X + 0.5, Z, dx=1) - sv(psxz, X - 1, Z) / (24 * h)
                            + sv(pszz, X, Z + 0.5, dz=1) - sv(pszz, X, Z - 1) / (24 * h))
    shape = (nx, nz)
    model = {k: np.full(shape, v, order="F") for k, v in c.items()}
    model["rho"] = np.full(shape, rho, order="F")
    for k in ("gamma_x", "gamma_z", "gamma_xz"):
        model[k] = np.zeros(shape, order="F")
    model.update(models._cpml_model(shape, cpml, (h, h), dt, 4000.0, 50.0))
    p = Problem(family=models.SEISMIC2, nx=nx, nz=nz, dx=h, dz=h, dt=dt, time_steps=1, cpml=cpml,
                xind=n // 2, zind=n // 2, model=model, src={}, fields0={"vx": vx0, "vz": vz0},
                receivers=np.zeros(1, dtype=np.int32), density="harmonic")
    m = np.zeros(shape, dtype=bool)
    lo, hi = cpml + 4, n + cpml - 4
    m[lo:hi, lo:hi] = True
    exp = {"vx": (vx1, vx0), "vz": (vz1, vz0), "sigmaxx": (sxx, 0.0), "sigmazz": (szz, 0.0), "sigmaxz": (sxz, 0.0)}
    return p, {k: (np.asfortranarray(v), m, np.max(np.abs((v - b)[m]))) for k, (v, b) in exp.items()}


def _shift_matrix(n: int, t: float) -> np.ndarray:
    """T with (T @ c) the coefficients of p(x + t) for p of coefficients c."""
    from math import comb
    T = np.zeros((n, n))
    for a in range(n):
        for a2 in range(a + 1):
            T[a2, a] = comb(a, a2) * t ** (a - a2)
    return T


def _shift(c: np.ndarray, shifts) -> np.ndarray:
    """Coefficients of p(x1 + t1, x2 + t2, ...) given those of p."""
    out = c
    for ax, t in enumerate(shifts):
        if t:
            out = np.moveaxis(np.tensordot(_shift_matrix(c.shape[ax], t), np.moveaxis(out, ax, 0), axes=1), 0, ax)
    return out


def _shift2(c: np.ndarray, sx: float, sz: float) -> np.ndarray:
    return _shift(c, (sx, sz))


# ------------------------------------------------------------------ 3D
def _poly3(rng, deg: int = 3) -> np.ndarray:
    c = np.zeros((deg + 1,) * 3)
    for a in range(deg + 1):
        for b in range(deg + 1 - a):
            for d in range(deg + 1 - a - b):
                c[a, b, d] = rng.uniform(-1.0, 1.0)
    return c


def _ev3(c, X, Y, Z, L, d=(0, 0, 0)):
    cc = c
    for ax, k in enumerate(d):
        if k:
            cc = P.polyder(cc, k, axis=ax)
    return P.polyval3d(X / L, Y / L, Z / L, cc) / L ** sum(d)


# Voigt rows of the six stresses (xx yy zz yz xz xy) in C21 names
def _c(i: int, j: int) -> str:
    a, b = min(i, j), max(i, j)
    return f"c{a}{b}"


# stress loops of seismic3 (cpmlfdtd.f08:1761-1992): the half-point side of
# each axis derivative (+1 forward, -1 backward) and the stresses they update
LOOPS3 = {1: ((+1, -1, -1), ("sigmaxx", "sigmayy", "sigmazz")), 2: ((-1, +1, -1), ("sigmaxy",)),
          3: ((-1, -1, +1), ("sigmaxz",)), 4: ((+1, +1, +1), ("sigmayz",))}
VOIGT_ROW = {"sigmaxx": 1, "sigmayy": 2, "sigmazz": 3, "sigmayz": 4, "sigmaxz": 5, "sigmaxy": 6}


def random_stiffness3(rng) -> dict:
    c = models.random_orthotropic(rng)
    R = models.euler_zxz(*rng.uniform(0, 2 * np.pi, 3))
    M = models.bond_matrix(R)
    cr = M @ c @ M.T
    cr = 0.5 * (cr + cr.T)
    return {_c(i + 1, j + 1): float(cr[i, j]) for i in range(6) for j in range(i, 6)}


def seismic3_manufactured(n: int = 24, cpml: int = 6, dt: float = 1e-3, rho: float = 2100.0, seed: int = 12,
                          nx_extra: int = 0):
    """3D counterpart of seismic2_manufactured: a homogeneous rotated
    orthotropic medium (21 C_ij), cubic velocities, one step."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n + nx_extra + 2 * cpml, n + 2 * cpml, n + 2 * cpml
    L = float(n)
    cv = [_poly3(rng) for _ in range(3)]   # vx vy vz
    C = random_stiffness3(rng)
    i = np.arange(nx, dtype=np.float64)[:, None, None]
    j = np.arange(ny, dtype=np.float64)[None, :, None]
    k = np.arange(nz, dtype=np.float64)[None, None, :]
    X, Y, Z = i + 0 * j + 0 * k, 0 * i + j + 0 * k, 0 * i + 0 * j + k
    v0 = [np.asfortranarray(_ev3(c, X, Y, Z, L)) for c in cv]

    def dpoly(f, ax, side):
        """coefficients (unit coordinates) of d v_f / d axis at the loop's half point"""
        d = P.polyder(cv[f], 1, axis=ax) / L
        d = np.pad(d, [(0, 4 - d.shape[a]) for a in range(3)])
        sh = [0.0, 0.0, 0.0]
        sh[ax] = 0.5 * side / L
        return _shift(d, sh)

    spoly = {}
    for _, (side, names) in LOOPS3.items():
        g = [[dpoly(f, ax, side[ax]) for ax in range(3)] for f in range(3)]
        # Voigt strain rates (engineering shears): xx yy zz yz xz xy
        e = [g[0][0], g[1][1], g[2][2], g[1][2] + g[2][1], g[0][2] + g[2][0], g[0][1] + g[1][0]]
        for nm in names:
            r = VOIGT_ROW[nm]
            spoly[nm] = dt * sum(C[_c(r, qq + 1)] * e[qq] for qq in range(6))
    sig = {nm: _ev3(c, X, Y, Z, L) for nm, c in spoly.items()}

    def q(nm, ax, side):
        """the reference's three-term form applied to a quadratic stress: the
        exact derivative at the half point plus its zeroth-order term"""
        d = [0, 0, 0]
        d[ax] = 1
        h = [0.0, 0.0, 0.0]
        h[ax] = 0.5 * side
        o = [0.0, 0.0, 0.0]
        o[ax] = -side  # backward (side -1) reads s(i+1), forward reads s(i-1)
        exact = _ev3(spoly[nm], X + h[0], Y + h[1], Z + h[2], L, tuple(d))
        term = _ev3(spoly[nm], X + o[0], Y + o[1], Z + o[2], L) / 24.0
        return exact + term if side < 0 else exact - term

    # velocity loops (:2014-2127)
    vx1 = v0[0] + dt / rho * (q("sigmaxx", 0, -1) + q("sigmaxy", 1, -1) + q("sigmaxz", 2, -1))
    vy1 = v0[1] + dt / rho * (q("sigmaxy", 0, +1) + q("sigmayy", 1, +1) + q("sigmayz", 2, -1))
    vz1 = v0[2] + dt / rho * (q("sigmaxz", 0, +1) + q("sigmayz", 1, -1) + q("sigmazz", 2, +1))
    shape = (nx, ny, nz)
    model = {nm: np.full(shape, C[nm], order="F") for nm in C21}
    model["rho"] = np.full(shape, rho, order="F")
    for nm in ("gamma_x", "gamma_y", "gamma_z", "gamma_xy", "gamma_yz", "gamma_xz"):
        model[nm] = np.zeros(shape, order="F")
    model.update(models._cpml_model(shape, cpml, (1.0, 1.0, 1.0), dt, 4000.0, 50.0))
    p = Problem(family=models.SEISMIC3, nx=nx, ny=ny, nz=nz, dx=1.0, dy=1.0, dz=1.0, dt=dt, time_steps=1,
                cpml=cpml, xind=n // 2, yind=n // 2, zind=n // 2, model=model, src={},
                fields0={"vx": v0[0], "vy": v0[1], "vz": v0[2]}, receivers=np.zeros(1, dtype=np.int32),
                density="harmonic")
    m = np.zeros(shape, dtype=bool)
    m[cpml + 4:nx - cpml - 4, cpml + 4:ny - cpml - 4, cpml + 4:nz - cpml - 4] = True
    exp = {"vx": (vx1, v0[0]), "vy": (vy1, v0[1]), "vz": (vz1, v0[2]), **{k: (v, 0.0) for k, v in sig.items()}}
    return p, {k: (np.asfortranarray(v), m, np.max(np.abs((v - b)[m]))) for k, (v, b) in exp.items()}


def check_manufactured(fields: list, names: list, expected: dict, rtol: float) -> dict:
    """Largest error of each checked field over its mask, relative to the
    largest change the step makes to that field (the stresses start at zero;
    for the velocities the step's change is far smaller than the velocity);
    asserts <= rtol."""
    out = {}
    for nm, got in zip(names, fields):
        if nm not in expected:
            continue
        want, m, scale = expected[nm]
        err = float(np.max(np.abs(np.asarray(got)[m] - want[m])) / scale)
        out[nm] = err
        assert err <= rtol, (nm, err)
    return out


# ------------------------------------------------------------------ EM
CLIGHT = models.CLIGHT


def electromag2_vacuum(n: int, cpml: int, nt: int, f0: float, src, rec_cells, comp: str = "z", h: float = 0.02,
                       eps=None, sig=None) -> Problem:
    """electromag2 with eps_r = 1, sigma = 0 (or the given padded grids), a
    Gaussian-derivative source on `comp` at interior cell `src`."""
    p = models.electromag2_blocks(n=n, cpml=cpml, nt=nt, h=h, f0=f0, src=src, nrec=2, rec_z=5, nblocks=0)
    shape = p.shape
    m = dict(p.model)
    one = np.full(shape, 1.0, order="F")
    m["e11"] = one if eps is None else eps
    m["e33"] = m["e11"].copy(order="F")
    m["s11"] = np.zeros(shape, order="F") if sig is None else sig
    m["s33"] = m["s11"].copy(order="F")
    dt = models.courant_dt(CLIGHT, (h, h))
    m.update(models._cpml_model(shape, cpml, (h, h), dt, CLIGHT, f0))
    return dataclasses.replace(p, model=m, dt=dt, src={comp: models.gaussian(nt, dt, f0, 1)},
                               receivers=np.asarray(rec_cells, dtype=np.int32))


def electromag3_vacuum(n: int, cpml: int, nt: int, f0: float, src, rec_cells, comp: str = "z",
                       h: float = 0.02) -> Problem:
    p = models.electromag3_blocks(n=n, cpml=cpml, nt=nt, h=h, f0=f0, nblocks=0)
    p = dataclasses.replace(p, xind=src[0], yind=src[1], zind=src[2])
    shape = p.shape
    m = dict(p.model)
    for nm in ("e11", "e22", "e33"):
        m[nm] = np.full(shape, 1.0, order="F")
    for nm in ("e12", "e13", "e23", "s11", "s12", "s13", "s22", "s23", "s33"):
        m[nm] = np.zeros(shape, order="F")
    dt = models.courant_dt(CLIGHT, (h, h, h))
    m.update(models._cpml_model(shape, cpml, (h, h, h), dt, CLIGHT, f0))
    return dataclasses.replace(p, model=m, dt=dt, src={comp: models.gaussian(nt, dt, f0, 1)},
                               receivers=np.asarray(rec_cells, dtype=np.int32))


def xcorr_lag(a: np.ndarray, b: np.ndarray, dt: float) -> float:
    """Delay of b behind a: the peak of their cross-correlation, refined by
    a parabola through its three highest samples."""
    c = np.correlate(b, a, "full")
    k = int(np.argmax(c))
    y0, y1, y2 = c[k - 1], c[k], c[k + 1]
    d = 0.5 * (y0 - y2) / (y0 - 2.0 * y1 + y2)
    return (k + d - (len(a) - 1)) * dt
