"""Seeded synthetic models of the benchmark configurations.

No public dataset exists for these solvers; the workloads are synthetic
models with the stated shapes, sizes and value ranges.  Every generator is
deterministic in its ``seed``.  Grids are padded (interior + 2*cpml per
axis) and filled by edge replication into the PML, the way the reference's
material pre-pass does (legacy/cpmlfdtd_cbindings.f95:439-536).

Time step rule: Courant number 0.5, ``dt = 0.5 / (vmax * sqrt(sum 1/h_i^2))``
with the reference's background speeds: elastic ``vmax = sqrt(max eig(C in
Mandel form) / min rho)`` (src/fortran/cpmlfdtd.f08:227-229), EM
``vmax = c / sqrt(min eps_r)`` (:2472-2475).
"""
from __future__ import annotations

import numpy as np

from ._lib import ELECTROMAG2, ELECTROMAG3, ELECTROMAG25, SEISMIC2, SEISMIC3, SEISMIC25
from .api import C21, Problem
from .cpml import cpml_grids

CLIGHT = 2.9979458e8  # constants.f08:8


# ------------------------------------------------------------------ wavelets
def ricker(nt: int, dt: float, f0: float, t0: float | None = None, amp: float = 1.0) -> np.ndarray:
    """(1 - 2a^2) exp(-a^2), a = pi f0 (t - t0), t0 = 1/f0 by default
    (legacy/plane_wave.f08:97-118); sample n is used at step n+1."""
    t = np.arange(nt) * dt
    t0 = 1.0 / f0 if t0 is None else t0
    a = np.pi * f0 * (t - t0)
    return amp * (1.0 - 2.0 * a * a) * np.exp(-a * a)


def gaussian(nt: int, dt: float, f0: float, order: int = 1, amp: float = 1.0) -> np.ndarray:
    """gaus0/gaus1/gaus2 of src/fortran/plane_wave_source.f08:141-161 (t0 = 1.5/f0)."""
    t = np.arange(nt) * dt
    a = np.pi * f0 * (t - 1.5 / f0)
    g = np.exp(-a * a)
    w = {0: g, 1: -2.0 * a * g, 2: (1.0 - 2.0 * a * a) * g}[order]
    return amp * w


# ------------------------------------------------------------------ helpers
def courant_dt(vmax: float, spacing, courant: float = 0.5) -> float:
    return courant / (vmax * np.sqrt(sum(1.0 / h ** 2 for h in spacing)))


def mandel2(c11, c13, c15, c33, c35, c55) -> np.ndarray:
    r2 = np.sqrt(2.0)
    return np.array([[c11, c13, r2 * c15], [c13, c33, r2 * c35], [r2 * c15, r2 * c35, 2.0 * c55]])


def voigt6(c: dict) -> np.ndarray:
    """6x6 Voigt matrix (order xx, yy, zz, yz, xz, xy) from c11..c66."""
    m = np.zeros((6, 6))
    for a in range(6):
        for b in range(a, 6):
            m[a, b] = m[b, a] = c[f"c{a + 1}{b + 1}"]
    return m


def mandel6(m: np.ndarray) -> np.ndarray:
    w = np.array([1, 1, 1, np.sqrt(2), np.sqrt(2), np.sqrt(2)])
    return m * np.outer(w, w)


def bond_matrix(R: np.ndarray) -> np.ndarray:
    """6x6 Bond stress-transformation matrix of rotation R (Voigt order)."""
    M = np.zeros((6, 6))
    pairs = [(0, 0), (1, 1), (2, 2), (1, 2), (2, 0), (0, 1)]
    for I, (i, j) in enumerate(pairs):
        for J, (k, l) in enumerate(pairs):
            if J < 3:
                M[I, J] = R[i, k] * R[j, l]
            else:
                M[I, J] = R[i, k] * R[j, l] + R[i, l] * R[j, k]
    return M


def euler_zxz(a: float, b: float, c: float) -> np.ndarray:
    def rz(t):
        return np.array([[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1]])

    def rx(t):
        return np.array([[1, 0, 0], [0, np.cos(t), -np.sin(t)], [0, np.sin(t), np.cos(t)]])

    return rz(a) @ rx(b) @ rz(c)


def pad_edge(a: np.ndarray, cpml: int) -> np.ndarray:
    return np.asfortranarray(np.pad(a, cpml, mode="edge"))


def _cpml_model(shape, cpml, spacing, dt, vmax, f0, kappa_max=2.0) -> dict:
    g = cpml_grids(shape, cpml, spacing, dt, vmax, f0, kappa_max)
    return {k: g[k] for k in ("kappa", "kappa_half", "acoef", "acoef_half", "bcoef", "bcoef_half")}


def _linspace_idx(lo: int, hi: int, n: int) -> np.ndarray:
    return np.rint(np.linspace(lo, hi, n)).astype(int)


# ------------------------------------------------------------------ seismic2
TWO_LAYER_TOP = dict(c11=8.0e9, c13=5.44e9, c15=0.0, c33=8.0e9, c35=0.0, c55=1.28e9, rho=2000.0)
TWO_LAYER_BOTTOM = dict(c11=14.1e9, c13=5.8e9, c15=0.0, c33=15.2e9, c35=0.0, c55=3.0e9, rho=917.0)


def seismic2_two_layer(n: int = 256, cpml: int = 20, nt: int = 2000, h: float = 1.0, f0: float = 60.0,
                       src=(128, 40), nrec: int = 64, rec_z: int = 20, interface: int | None = None,
                       density: str = "arithmetic", anomaly: dict | None = None, gamma: float = 0.0,
                       dt: float | None = None) -> Problem:
    """2D P-SV two-layer model (isotropic over ice-like VTI), vertical-force
    Ricker source, a line of receivers.  Defaults are the 256^2 benchmark
    case; tests use smaller ``n``.  ``anomaly`` = dict(x, z, sigma, frac)
    adds a Gaussian perturbation of c11, c33, c55 (the FWI target model)."""
    nx = nz = n
    interface = n // 2 if interface is None else interface
    zz = np.arange(nz)[None, :]
    xx = np.arange(nx)[:, None]
    top = np.broadcast_to(zz < interface, (nx, nz))
    mod = {}
    for k in ("c11", "c13", "c15", "c33", "c35", "c55", "rho"):
        mod[k] = np.where(top, TWO_LAYER_TOP[k], TWO_LAYER_BOTTOM[k]).astype(np.float64)
    if anomaly:
        g = np.exp(-((xx - anomaly["x"]) ** 2 + (zz - anomaly["z"]) ** 2) / (2.0 * anomaly["sigma"] ** 2))
        for k in ("c11", "c33", "c55"):
            mod[k] = mod[k] * (1.0 + anomaly["frac"] * g)
    vmax = 0.0
    for lay in (TWO_LAYER_TOP, TWO_LAYER_BOTTOM):
        ev = np.linalg.eigvalsh(mandel2(lay["c11"], lay["c13"], lay["c15"], lay["c33"], lay["c35"], lay["c55"]))
        vmax = max(vmax, np.sqrt(ev.max() / min(TWO_LAYER_TOP["rho"], TWO_LAYER_BOTTOM["rho"])))
    if anomaly:
        vmax *= np.sqrt(1.0 + anomaly["frac"])
    dt = courant_dt(vmax, (h, h)) if dt is None else dt
    model = {k: pad_edge(v, cpml) for k, v in mod.items()}
    for k in ("gamma_x", "gamma_z", "gamma_xz"):
        model[k] = np.full_like(model["rho"], gamma, order="F")
    shape = (nx + 2 * cpml, nz + 2 * cpml)
    model.update(_cpml_model(shape, cpml, (h, h), dt, vmax, f0))
    rx = _linspace_idx(1, n, nrec)
    rec = (rx + cpml - 1) + shape[0] * (rec_z + cpml - 1)
    return Problem(family=SEISMIC2, nx=shape[0], nz=shape[1], dx=h, dz=h, dt=dt, time_steps=nt, cpml=cpml,
                   xind=src[0], zind=src[1], model=model, src={"z": ricker(nt, dt, f0)},
                   receivers=rec.astype(np.int32), density=density,
                   meta={"vmax": vmax, "f0": f0, "config": "seismic2 two-layer"})


# --------------------------------------------------------------- electromag2
def electromag2_blocks(n: int = 1024, cpml: int = 20, nt: int = 4000, h: float = 0.02, f0: float = 100e6,
                       src=(512, 30), nrec: int = 128, rec_z: int = 25, nblocks: int = 12,
                       seed: int = 1) -> Problem:
    """2D GPR model: background eps_r = 4, sigma = 1e-4 S/m, ``nblocks`` seeded
    rectangles with diagonal eps_xx, eps_zz ~ U[3, 25] and sigma ~ U[0, 0.01]
    (sigma_11 = sigma_33, eps_13 = sigma_13 = 0); Gaussian-derivative source."""
    rng = np.random.default_rng(seed)
    nx = nz = n
    e11 = np.full((nx, nz), 4.0)
    e33 = np.full((nx, nz), 4.0)
    sig = np.full((nx, nz), 1.0e-4)
    for _ in range(nblocks):
        x0, z0 = rng.integers(0, n - n // 8, size=2)
        wx, wz = rng.integers(n // 32 + 1, n // 4 + 2, size=2)
        exx, ezz = rng.uniform(3.0, 25.0, size=2)
        s = rng.uniform(0.0, 0.01)
        e11[x0:x0 + wx, z0:z0 + wz] = exx
        e33[x0:x0 + wx, z0:z0 + wz] = ezz
        sig[x0:x0 + wx, z0:z0 + wz] = s
    emin = min(e11.min(), e33.min())
    vmax = CLIGHT / np.sqrt(emin)
    dt = courant_dt(vmax, (h, h))
    shape = (nx + 2 * cpml, nz + 2 * cpml)
    model = {"e11": pad_edge(e11, cpml), "e13": np.zeros(shape, order="F"), "e33": pad_edge(e33, cpml),
             "s11": pad_edge(sig, cpml), "s13": np.zeros(shape, order="F"), "s33": pad_edge(sig, cpml)}
    model.update(_cpml_model(shape, cpml, (h, h), dt, vmax, f0))
    rx = _linspace_idx(1, n, nrec)
    rec = (rx + cpml - 1) + shape[0] * (rec_z + cpml - 1)
    return Problem(family=ELECTROMAG2, nx=shape[0], nz=shape[1], dx=h, dz=h, dt=dt, time_steps=nt, cpml=cpml,
                   xind=src[0], zind=src[1], model=model, src={"x": gaussian(nt, dt, f0, 1), "z": gaussian(nt, dt, f0, 1)},
                   receivers=rec.astype(np.int32), meta={"vmax": vmax, "f0": f0, "seed": seed,
                                                         "config": "electromag2 blocks"})


# ------------------------------------------------------------------ seismic3
def random_orthotropic(rng) -> np.ndarray:
    """Positive-definite orthotropic 6x6 Voigt stiffness in the stated ranges."""
    while True:
        c = np.zeros((6, 6))
        c[0, 0], c[1, 1], c[2, 2] = rng.uniform(8e9, 16e9, 3)
        c[0, 1], c[0, 2], c[1, 2] = rng.uniform(3e9, 6e9, 3)
        c[1, 0], c[2, 0], c[2, 1] = c[0, 1], c[0, 2], c[1, 2]
        c[3, 3], c[4, 4], c[5, 5] = rng.uniform(1e9, 4e9, 3)
        if np.linalg.eigvalsh(c).min() > 0:
            return c


def seismic3_layers(n: int = 320, cpml: int = 16, nt: int = 1500, h: float = 1.0, f0: float = 40.0,
                    nlayers: int = 5, seed: int = 2, nrec_side: int = 32, rec_z: int = 4,
                    src_z: int = 8, ny: int | None = None, nz: int | None = None,
                    density: str = "arithmetic") -> Problem:
    """3D model of ``nlayers`` horizontal layers, each an orthotropic stiffness
    rotated by seeded Euler angles into a full 21-component C_ij, rho ~
    U[900, 2600], gamma_x,y,z ~ U[0, 50] (shear gammas: mean of their two
    axes); vertical Ricker force at the centre-top; a square receiver grid."""
    rng = np.random.default_rng(seed)
    nx = n
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    bounds = np.linspace(0, nz, nlayers + 1).astype(int)
    layers = []
    for _ in range(nlayers):
        c = random_orthotropic(rng)
        R = euler_zxz(*rng.uniform(0, 2 * np.pi, 3))
        M = bond_matrix(R)
        cr = M @ c @ M.T
        cr = 0.5 * (cr + cr.T)
        gx, gy, gz = rng.uniform(0.0, 50.0, 3)
        layers.append({"C": cr, "rho": rng.uniform(900.0, 2600.0),
                       "gamma": (gx, gy, gz, 0.5 * (gx + gy), 0.5 * (gy + gz), 0.5 * (gx + gz))})
    rho_min = min(L["rho"] for L in layers)
    vmax = max(np.sqrt(np.linalg.eigvalsh(mandel6(L["C"])).max() / rho_min) for L in layers)
    dt = courant_dt(vmax, (h, h, h))
    shape = (nx + 2 * cpml, ny + 2 * cpml, nz + 2 * cpml)
    # layer index per padded z (edge replication into the PML)
    zl = np.clip(np.arange(shape[2]) - cpml, 0, nz - 1)
    lid = np.searchsorted(bounds[1:], zl, side="right")
    model = {}

    def layered(vals):
        a = np.empty(shape, order="F")
        for L in range(nlayers):
            a[:, :, lid == L] = vals[L]
        return a

    for idx, name in enumerate(C21):
        i, j = int(name[1]) - 1, int(name[2]) - 1
        model[name] = layered([L["C"][i, j] for L in layers])
    model["rho"] = layered([L["rho"] for L in layers])
    for q, name in enumerate(("gamma_x", "gamma_y", "gamma_z", "gamma_xy", "gamma_yz", "gamma_xz")):
        model[name] = layered([L["gamma"][q] for L in layers])
    model.update(_cpml_model(shape, cpml, (h, h, h), dt, vmax, f0))
    rx = _linspace_idx(1, nx, nrec_side)
    ry = _linspace_idx(1, ny, nrec_side)
    RX, RY = np.meshgrid(rx, ry, indexing="ij")
    rec = (RX.ravel() + cpml - 1) + shape[0] * ((RY.ravel() + cpml - 1) + shape[1] * (rec_z + cpml - 1))
    return Problem(family=SEISMIC3, nx=shape[0], ny=shape[1], nz=shape[2], dx=h, dy=h, dz=h, dt=dt,
                   time_steps=nt, cpml=cpml, xind=nx // 2, yind=ny // 2, zind=src_z, model=model,
                   src={"z": ricker(nt, dt, f0)}, receivers=rec.astype(np.int32), density=density,
                   meta={"vmax": vmax, "f0": f0, "seed": seed, "config": "seismic3 layers"})


# ------------------------------------------------------------------ 2.5D
def seismic25_two_layer(n: int = 128, cpml: int = 10, nt: int = 400, h: float = 1.0, f0: float = 60.0,
                        ky: float = 0.05, seed: int = 3, nrec: int = 32, density: str = "harmonic") -> Problem:
    """2.5D elastic model: the two-layer stiffness of the 2D case rotated into
    a full 21-component C_ij per layer, complex fields with d/dy = i ky."""
    rng = np.random.default_rng(seed)
    nx = nz = n
    lay = []
    for base in (TWO_LAYER_TOP, TWO_LAYER_BOTTOM):
        c = np.zeros((6, 6))
        c[0, 0] = c[1, 1] = base["c11"]
        c[2, 2] = base["c33"]
        c[0, 2] = c[2, 0] = c[1, 2] = c[2, 1] = base["c13"]
        c[0, 1] = c[1, 0] = base["c11"] - 2 * base["c55"]
        c[3, 3] = c[4, 4] = base["c55"]
        c[5, 5] = base["c55"]
        M = bond_matrix(euler_zxz(*rng.uniform(0, 0.5, 3)))
        cr = M @ c @ M.T
        lay.append((0.5 * (cr + cr.T), base["rho"]))
    zz = np.arange(nz)[None, :]
    top = np.broadcast_to(zz < nz // 2, (nx, nz))
    model = {}
    for name in C21:
        i, j = int(name[1]) - 1, int(name[2]) - 1
        model[name] = pad_edge(np.where(top, lay[0][0][i, j], lay[1][0][i, j]), cpml)
    model["rho"] = pad_edge(np.where(top, lay[0][1], lay[1][1]), cpml)
    g = rng.uniform(0, 20, 6)
    for q, name in enumerate(("gamma_x", "gamma_y", "gamma_z", "gamma_xy", "gamma_yz", "gamma_xz")):
        model[name] = np.full_like(model["rho"], g[q], order="F")
    vmax = max(np.sqrt(np.linalg.eigvalsh(mandel6(c)).max() / min(r for _, r in lay)) for c, _ in lay)
    dt = courant_dt(vmax, (h, h))
    shape = (nx + 2 * cpml, nz + 2 * cpml)
    model.update(_cpml_model(shape, cpml, (h, h), dt, vmax, f0))
    rx = _linspace_idx(1, n, nrec)
    rec = (rx + cpml - 1) + shape[0] * (n // 8 + cpml - 1)
    w = ricker(nt, dt, f0)
    return Problem(family=SEISMIC25, nx=shape[0], nz=shape[1], dx=h, dz=h, dt=dt, time_steps=nt, cpml=cpml,
                   xind=n // 2, zind=n // 4, model=model, src={"x": 0.3 * w, "y": 0.5 * w, "z": w},
                   receivers=rec.astype(np.int32), ky=ky, density=density,
                   meta={"vmax": vmax, "f0": f0, "seed": seed, "config": "seismic25 two-layer"})


def electromag25_blocks(n: int = 128, cpml: int = 10, nt: int = 400, h: float = 0.02, f0: float = 100e6,
                        ky: float = 2.0, seed: int = 4, nblocks: int = 6, nrec: int = 32) -> Problem:
    """2.5D GPR model with full symmetric eps and sigma tensors per block."""
    rng = np.random.default_rng(seed)
    nx = nz = n
    comps = ("11", "12", "13", "22", "23", "33")
    eps = {c: np.full((nx, nz), 4.0 if c[0] == c[1] else 0.0) for c in comps}
    sig = {c: np.full((nx, nz), 1.0e-4 if c[0] == c[1] else 0.0) for c in comps}
    for _ in range(nblocks):
        x0, z0 = rng.integers(0, n - n // 8, size=2)
        wx, wz = rng.integers(n // 16 + 1, n // 3, size=2)
        d = rng.uniform(3.0, 25.0, 3)
        off = rng.uniform(-0.3, 0.3, 3) * min(d)
        e = {"11": d[0], "22": d[1], "33": d[2], "12": off[0], "13": off[1], "23": off[2]}
        s = {"11": rng.uniform(0, 0.01), "22": rng.uniform(0, 0.01), "33": rng.uniform(0, 0.01),
             "12": 0.0, "13": 0.0, "23": 0.0}
        for c in comps:
            eps[c][x0:x0 + wx, z0:z0 + wz] = e[c]
            sig[c][x0:x0 + wx, z0:z0 + wz] = s[c]
    emin = min(eps[c].min() for c in ("11", "22", "33")) * 0.7
    vmax = CLIGHT / np.sqrt(emin)
    dt = courant_dt(vmax, (h, h))
    shape = (nx + 2 * cpml, nz + 2 * cpml)
    model = {}
    for c in comps:
        model["e" + c] = pad_edge(eps[c], cpml)
        model["s" + c] = pad_edge(sig[c], cpml)
    model.update(_cpml_model(shape, cpml, (h, h), dt, vmax, f0))
    rx = _linspace_idx(1, n, nrec)
    rec = (rx + cpml - 1) + shape[0] * (n // 8 + cpml - 1)
    w = gaussian(nt, dt, f0, 1)
    return Problem(family=ELECTROMAG25, nx=shape[0], nz=shape[1], dx=h, dz=h, dt=dt, time_steps=nt, cpml=cpml,
                   xind=n // 2, zind=n // 4, model=model, src={"x": w, "y": 0.5 * w, "z": 0.25 * w},
                   receivers=rec.astype(np.int32), ky=ky,
                   meta={"vmax": vmax, "f0": f0, "seed": seed, "config": "electromag25 blocks"})


def electromag3_blocks(n: int = 96, cpml: int = 10, nt: int = 300, h: float = 0.02, f0: float = 100e6,
                       seed: int = 6, nblocks: int = 6, nrec_side: int = 16, ny: int | None = None,
                       nz: int | None = None) -> Problem:
    """3D GPR model: a background of eps = 4, sigma = 1e-4 with ``nblocks``
    seeded boxes, each with its own full symmetric eps tensor (diagonal
    U[3, 25], off-diagonal up to 30% of the smallest diagonal) and diagonal
    sigma U[0, 0.01]; a Gaussian-derivative point source driving all three E
    components at the centre, a square receiver grid near the top."""
    rng = np.random.default_rng(seed)
    nx = n
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    comps = ("11", "12", "13", "22", "23", "33")
    eps = {c: np.full((nx, ny, nz), 4.0 if c[0] == c[1] else 0.0) for c in comps}
    sig = {c: np.full((nx, ny, nz), 1.0e-4 if c[0] == c[1] else 0.0) for c in comps}
    dims = np.array([nx, ny, nz])
    for _ in range(nblocks):
        lo = rng.integers(0, dims - dims // 8)
        w = rng.integers(dims // 16 + 1, dims // 3)
        d = rng.uniform(3.0, 25.0, 3)
        off = rng.uniform(-0.3, 0.3, 3) * min(d)
        e = {"11": d[0], "22": d[1], "33": d[2], "12": off[0], "13": off[1], "23": off[2]}
        sd = rng.uniform(0, 0.01, 3)
        s = {"11": sd[0], "22": sd[1], "33": sd[2], "12": 0.0, "13": 0.0, "23": 0.0}
        box = tuple(slice(lo[q], lo[q] + w[q]) for q in range(3))
        for c in comps:
            eps[c][box] = e[c]
            sig[c][box] = s[c]
    emin = min(eps[c].min() for c in ("11", "22", "33")) * 0.7
    vmax = CLIGHT / np.sqrt(emin)
    dt = courant_dt(vmax, (h, h, h))
    shape = (nx + 2 * cpml, ny + 2 * cpml, nz + 2 * cpml)
    model = {}
    for c in comps:
        model["e" + c] = pad_edge(eps[c], cpml)
        model["s" + c] = pad_edge(sig[c], cpml)
    model.update(_cpml_model(shape, cpml, (h, h, h), dt, vmax, f0))
    rx = _linspace_idx(1, nx, nrec_side)
    ry = _linspace_idx(1, ny, nrec_side)
    RX, RY = np.meshgrid(rx, ry, indexing="ij")
    rec = (RX.ravel() + cpml - 1) + shape[0] * ((RY.ravel() + cpml - 1) + shape[1] * (nz // 8 + cpml - 1))
    w = gaussian(nt, dt, f0, 1)
    return Problem(family=ELECTROMAG3, nx=shape[0], ny=shape[1], nz=shape[2], dx=h, dy=h, dz=h, dt=dt,
                   time_steps=nt, cpml=cpml, xind=nx // 2, yind=ny // 2, zind=nz // 2, model=model,
                   src={"x": w, "y": 0.5 * w, "z": 0.25 * w}, receivers=rec.astype(np.int32),
                   meta={"vmax": vmax, "f0": f0, "seed": seed, "config": "electromag3 blocks"})


# ------------------------------------------------------------ ragged batch
def batch_layered_vti(nmodels: int = 64, nt: int = 3000, cpml: int = 20, seed: int = 5, nmin: int = 256,
                      nmax: int = 1024, step: int = 32, nrec: int = 64, h: float = 1.0) -> list:
    """The ragged multi-model workload: ``nmodels`` 2D elastic models with nx,
    nz drawn uniformly from [nmin, nmax] in multiples of ``step``, each a
    stack of 2-5 VTI layers with stiffness and density drawn from the ranges
    of the two-layer model, its own Ricker source (f0 ~ U[30, 90] Hz) at a
    random position in the top 20%, and ``nrec`` receivers; every model keeps
    its own Courant-0.5 time step."""
    rng = np.random.default_rng(seed)
    out = []
    sizes = np.arange(nmin, nmax + 1, step)
    lo = {k: min(TWO_LAYER_TOP[k], TWO_LAYER_BOTTOM[k]) for k in TWO_LAYER_TOP}
    hi = {k: max(TWO_LAYER_TOP[k], TWO_LAYER_BOTTOM[k]) for k in TWO_LAYER_TOP}
    for m in range(nmodels):
        nx, nz = int(rng.choice(sizes)), int(rng.choice(sizes))
        nl = int(rng.integers(2, 6))
        bounds = np.sort(rng.choice(np.arange(1, nz), size=nl - 1, replace=False)) if nl > 1 else []
        lid = np.searchsorted(bounds, np.arange(nz), side="right")
        lay = []
        for _ in range(nl):
            d = {k: rng.uniform(lo[k], hi[k]) for k in ("c11", "c33", "c55", "rho")}
            d["c13"] = rng.uniform(lo["c13"], hi["c13"])
            d["c15"] = d["c35"] = 0.0
            lay.append(d)
        mod = {k: np.empty((nx, nz)) for k in ("c11", "c13", "c15", "c33", "c35", "c55", "rho")}
        for k in mod:
            mod[k][:, :] = np.array([lay[L][k] for L in lid])[None, :]
        rho_min = min(L["rho"] for L in lay)
        vmax = max(np.sqrt(np.linalg.eigvalsh(mandel2(L["c11"], L["c13"], 0.0, L["c33"], 0.0, L["c55"])).max() / rho_min)
                   for L in lay)
        dt = courant_dt(vmax, (h, h))
        f0 = float(rng.uniform(30.0, 90.0))
        model = {k: pad_edge(v, cpml) for k, v in mod.items()}
        for k in ("gamma_x", "gamma_z", "gamma_xz"):
            model[k] = np.zeros_like(model["rho"], order="F")
        shape = (nx + 2 * cpml, nz + 2 * cpml)
        model.update(_cpml_model(shape, cpml, (h, h), dt, vmax, f0))
        sx = int(rng.integers(1, nx + 1))
        sz = int(rng.integers(1, max(2, nz // 5) + 1))
        rx = _linspace_idx(1, nx, nrec)
        rec = (rx + cpml - 1) + shape[0] * (max(1, nz // 10) + cpml - 1)
        out.append(Problem(family=SEISMIC2, nx=shape[0], nz=shape[1], dx=h, dz=h, dt=dt, time_steps=nt, cpml=cpml,
                           xind=sx, zind=sz, model=model, src={"z": ricker(nt, dt, f0)},
                           receivers=rec.astype(np.int32),
                           meta={"vmax": vmax, "f0": f0, "seed": seed, "config": "ragged batch"}))
    return out
