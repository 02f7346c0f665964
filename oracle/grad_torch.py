"""FP64 gradient oracle for the 2D elastic misfit -- TEST INFRASTRUCTURE.

Only tests import this module.  It restates the seismic2 time loop of
src/fortran/cpmlfdtd.f08:311-576 (the statements of oracle_seismic2 in
oracle.c, here as whole-array torch expressions: the four loops in their
reference order, the three-term velocity stencils, the force source without
dt, the Dirichlet ring) so that torch.autograd gives, in FP64, the gradient
of

    L = 1/2 sum_shots sum_steps sum_receivers (vx - dx)^2 + (vz - dz)^2

with respect to c11, c13, c33, c55 and rho.  Its forward traces are checked
against oracle.c before its gradients are trusted.  Arrays are (nx, nz) with
x first, matching the Fortran-order grids of the reference.
"""
from __future__ import annotations

import numpy as np
import torch


def _mean(a, b, code):
    # averaging.f08:5-25
    if code == 1:
        return 2.0 * a * b / (a + b)
    if code == 2:
        return torch.sqrt(a * b)
    if code == 3:
        return 0.5 * (a + b)
    return a


def forward_traces(m: dict, dx: float, dz: float, dt: float, nt: int, src_cell: tuple, srcz,
                   rec: np.ndarray, density_code: int) -> torch.Tensor:
    """Receiver traces [nt][2][nrec] of one shot; ``m`` holds (nx, nz) FP64
    tensors (c11 c13 c15 c33 c35 c55 rho gamma_x gamma_z gamma_xz kappa
    kappa_half acoef acoef_half bcoef bcoef_half); ``src_cell`` = 0-based
    (i, k) of the force; ``rec`` = 0-based x-fastest linear cell indices."""
    c11, c13, c15, c33, c35, c55, rho = (m[k] for k in ("c11", "c13", "c15", "c33", "c35", "c55", "rho"))
    gx, gz, gxz = m["gamma_x"], m["gamma_z"], m["gamma_xz"]
    kap, kaph, ac, ach, bc, bch = (m[k] for k in ("kappa", "kappa_half", "acoef", "acoef_half", "bcoef",
                                                  "bcoef_half"))
    nx, nz = rho.shape
    z = torch.zeros_like(rho)
    vx, vz, sxx, szz, sxz = z, z, z, z, z
    mem = [z] * 12
    ri = torch.as_tensor(rec % nx, dtype=torch.long)
    rk = torch.as_tensor(rec // nx, dtype=torch.long)
    hx, hz = 24.0 * dx, 24.0 * dz
    isrc, ksrc = src_cell
    srcz = torch.as_tensor(np.asarray(srcz, dtype=np.float64))

    def S(a, I, K, di=0, dk=0):
        return a[I[0] + di:I[1] + di, K[0] + dk:K[1] + dk]

    def put(a, I, K, val):
        out = a.clone()
        out[I[0]:I[1], K[0]:K[1]] = val
        return out

    # 0-based half-open ranges of the four loops
    IN, KN = (1, nx - 2), (2, nz - 1)   # normal stresses: i 2..nx-2, j 3..nz-1 (1-based)
    IS, KS = (2, nx - 1), (1, nz - 2)   # shear stress:    i 3..nx-1, j 2..nz-2
    IX, KX = (2, nx - 1), (2, nz - 1)   # vx:              i 3..nx-1, j 3..nz-1
    IZ, KZ = (1, nx - 2), (1, nz - 2)   # vz:              i 2..nx-2, j 2..nz-2
    out = []
    for it in range(nt):
        # ---- normal stresses (cpmlfdtd.f08:324-353)
        I, K = IN, KN
        dvx_dx = (27.0 * (S(vx, I, K, 1) - S(vx, I, K)) - (S(vx, I, K, 2) - S(vx, I, K, -1))) / hx
        dvz_dz = (27.0 * (S(vz, I, K) - S(vz, I, K, 0, -1)) - (S(vz, I, K, 0, 1) - S(vz, I, K, 0, -2))) / hz
        dvz_dx = (27.0 * (S(vz, I, K, 1) - S(vz, I, K)) - (S(vz, I, K, 2) - S(vz, I, K, -1))) / hx
        dvx_dz = (27.0 * (S(vx, I, K) - S(vx, I, K, 0, -1)) - (S(vx, I, K, 0, 1) - S(vx, I, K, 0, -2))) / hz
        m0 = S(bch, I, K) * S(mem[0], I, K) + S(ach, I, K) * dvx_dx
        m1 = S(bch, I, K) * S(mem[1], I, K) + S(ach, I, K) * dvx_dz
        m3 = S(bc, I, K) * S(mem[3], I, K) + S(ac, I, K) * dvz_dz
        m2 = S(bc, I, K) * S(mem[2], I, K) + S(ac, I, K) * dvz_dx
        mem[0], mem[1], mem[2], mem[3] = put(mem[0], I, K, m0), put(mem[1], I, K, m1), put(mem[2], I, K, m2), \
            put(mem[3], I, K, m3)
        dvx_dx = dvx_dx / S(kaph, I, K) + m0
        dvx_dz = dvx_dz / S(kaph, I, K) + m1
        dvz_dz = dvz_dz / S(kap, I, K) + m3
        dvz_dx = dvz_dx / S(kap, I, K) + m2
        nsxx = (S(sxx, I, K) + (S(c11, I, K) * dvx_dx + S(c13, I, K) * dvz_dz + S(c15, I, K) * (dvz_dx + dvx_dz))
                * dt) / (1.0 + S(gx, I, K) * dt)
        nszz = (S(szz, I, K) + (S(c13, I, K) * dvx_dx + S(c33, I, K) * dvz_dz + S(c35, I, K) * (dvz_dx + dvx_dz))
                * dt) / (1.0 + S(gz, I, K) * dt)
        sxx, szz = put(sxx, I, K, nsxx), put(szz, I, K, nszz)
        # ---- shear stress (cpmlfdtd.f08:362-386)
        I, K = IS, KS
        dvx_dx = (27.0 * (S(vx, I, K) - S(vx, I, K, -1)) - (S(vx, I, K, 1) - S(vx, I, K, -2))) / hx
        dvz_dz = (27.0 * (S(vz, I, K, 0, 1) - S(vz, I, K)) - (S(vz, I, K, 0, 2) - S(vz, I, K, 0, -1))) / hz
        dvz_dx = (27.0 * (S(vz, I, K) - S(vz, I, K, -1)) - (S(vz, I, K, 1) - S(vz, I, K, -2))) / hx
        dvx_dz = (27.0 * (S(vx, I, K, 0, 1) - S(vx, I, K)) - (S(vx, I, K, 0, 2) - S(vx, I, K, 0, -1))) / hz
        m4 = S(bch, I, K) * S(mem[4], I, K) + S(ach, I, K) * dvx_dx
        m5 = S(bch, I, K) * S(mem[5], I, K) + S(ach, I, K) * dvx_dz
        m7 = S(bch, I, K) * S(mem[7], I, K) + S(ach, I, K) * dvz_dz
        m6 = S(bch, I, K) * S(mem[6], I, K) + S(ach, I, K) * dvz_dx
        mem[4], mem[5], mem[6], mem[7] = put(mem[4], I, K, m4), put(mem[5], I, K, m5), put(mem[6], I, K, m6), \
            put(mem[7], I, K, m7)
        dvx_dx = dvx_dx / S(kaph, I, K) + m4
        dvx_dz = dvx_dz / S(kaph, I, K) + m5
        dvz_dz = dvz_dz / S(kaph, I, K) + m7
        dvz_dx = dvz_dx / S(kaph, I, K) + m6
        nsxz = (S(sxz, I, K) + (S(c15, I, K) * dvx_dx + S(c35, I, K) * dvz_dz + S(c55, I, K) * (dvz_dx + dvx_dz))
                * dt) / (1.0 + S(gxz, I, K) * dt)
        sxz = put(sxz, I, K, nsxz)
        # ---- vx (cpmlfdtd.f08:399-416), three-term stencils
        I, K = IX, KX
        rhoxx = _mean(S(rho, I, K), S(rho, I, K, -1), density_code)
        rhozx = _mean(S(rho, I, K), S(rho, I, K, 0, -1), density_code)
        dsxx_dx = (27.0 * S(sxx, I, K) - 27.0 * S(sxx, I, K, -1) + S(sxx, I, K, -2)) / hx
        dsxz_dz = (27.0 * S(sxz, I, K) - 27.0 * S(sxz, I, K, 0, -1) + S(sxz, I, K, 0, -2)) / hz
        m8 = S(bc, I, K) * S(mem[8], I, K) + S(ac, I, K) * dsxx_dx
        m11 = S(bc, I, K) * S(mem[11], I, K) + S(ac, I, K) * dsxz_dz
        mem[8], mem[11] = put(mem[8], I, K, m8), put(mem[11], I, K, m11)
        dsxx_dx = dsxx_dx / S(kap, I, K) + m8
        dsxz_dz = dsxz_dz / S(kap, I, K) + m11
        vx = put(vx, I, K, S(vx, I, K) + dt * (dsxx_dx / rhoxx + dsxz_dz / rhozx))
        # ---- vz (cpmlfdtd.f08:428-446)
        I, K = IZ, KZ
        rhoxz = _mean(S(rho, I, K), S(rho, I, K, 1), density_code)
        rhozz = _mean(S(rho, I, K), S(rho, I, K, 0, 1), density_code)
        dsxz_dx = (-27.0 * S(sxz, I, K) + 27.0 * S(sxz, I, K, 1) - S(sxz, I, K, 2)) / hx
        dszz_dz = (-27.0 * S(szz, I, K) + 27.0 * S(szz, I, K, 0, 1) - S(szz, I, K, 0, 2)) / hz
        m10 = S(bch, I, K) * S(mem[10], I, K) + S(ach, I, K) * dsxz_dx
        m9 = S(bch, I, K) * S(mem[9], I, K) + S(ach, I, K) * dszz_dz
        mem[10], mem[9] = put(mem[10], I, K, m10), put(mem[9], I, K, m9)
        dsxz_dx = dsxz_dx / S(kaph, I, K) + m10
        dszz_dz = dszz_dz / S(kaph, I, K) + m9
        vz = put(vz, I, K, S(vz, I, K) + dt * (dsxz_dx / rhoxz + dszz_dz / rhozz))
        # ---- force source without dt (cpmlfdtd.f08:522-523)
        vz = vz.clone()
        vz[isrc, ksrc] = vz[isrc, ksrc] + srcz[it] / rho[isrc, ksrc]
        # ---- Dirichlet ring (cpmlfdtd.f08:534-549)
        ring = torch.ones_like(rho)
        ring[0, :] = 0.0
        ring[-1, :] = 0.0
        ring[:, 0] = 0.0
        ring[:, -1] = 0.0
        vx, vz = vx * ring, vz * ring
        out.append(torch.stack([vx[ri, rk], vz[ri, rk]]))
    return torch.stack(out)


def misfit_and_gradient(problem, shots, observed, density_code: int,
                        keys=("c11", "c13", "c33", "c55", "rho")):
    """FP64 L and dL/d{keys} ((nx, nz) numpy arrays; any seismic2 model slot,
    e.g. c15 and c35 as well) for a seismic2 Problem and the same shot list
    the GPU adjoint takes."""
    m = {k: torch.tensor(np.asarray(v, dtype=np.float64), requires_grad=k in keys) for k, v in problem.model.items()}
    rec = np.asarray(problem.receivers, dtype=np.int64)
    loss = torch.zeros((), dtype=torch.float64)
    for s, shot in enumerate(shots):
        tr = forward_traces(m, problem.dx, problem.dz, problem.dt, problem.time_steps,
                            (shot.xind + problem.cpml - 1, shot.zind + problem.cpml - 1), shot.srcz, rec,
                            density_code)
        obs = torch.as_tensor(np.asarray(observed[s], dtype=np.float64).reshape(tr.shape))
        loss = loss + 0.5 * ((tr - obs) ** 2).sum()
    loss.backward()
    return float(loss.detach()), {k: m[k].grad.numpy().copy() for k in keys}


# ---------------------------------------------------------------- electromag2
EPS0 = 8.85418782e-12                       # constants.f08
MU0 = 4.0 * 3.141592653589793238462643 * 1.0e-7
EM_KEYS = ("e11", "e13", "e33", "s11", "s13", "s33")


def em2_forward_traces(m: dict, dx: float, dz: float, dt: float, nt: int, src_cell: tuple, srcz,
                       rec: np.ndarray) -> torch.Tensor:
    """Receiver traces [nt][2][nrec] (Ex, Ez) of one electromag2 shot whose
    source drives Ez; the statements of oracle_electromag2 in oracle.c
    (cpmlfdtd.f08:2519-2748: eps scaled by eps0, det clamped at 1e-18 eps0^2,
    H then E update, Ez += f dt / eps33, ring on Ex, Ez, Hy) as torch
    expressions on (nx, nz) FP64 tensors."""
    e11, e13, e33 = m["e11"] * EPS0, m["e13"] * EPS0, m["e33"] * EPS0
    s11, s13, s33 = m["s11"], m["s13"], m["s33"]
    kap, kaph, ac, ach, bc, bch = (m[k] for k in ("kappa", "kappa_half", "acoef", "acoef_half", "bcoef",
                                                  "bcoef_half"))
    det = e11 * e33 - e13 * e13
    floor = 1.0e-18 * EPS0 * EPS0
    det = torch.where(det <= floor, torch.full_like(det, floor), det)
    aEx, bEx = e33 / det, -e13 / det
    dEx, eEx = (e33 * s11 - e13 * s13) / det, (e33 * s13 - e13 * s33) / det
    aEz, bEz = -e13 / det, e11 / det
    dEz, eEz = (e11 * s13 - e13 * s11) / det, (e11 * s33 - e13 * s13) / det
    dbHy = dt / MU0
    nx, nz = e11.shape
    z = torch.zeros_like(e11)
    Ex, Ez, Hy = z, z, z
    m0, m1, m2, m3 = z, z, z, z
    ri = torch.as_tensor(rec % nx, dtype=torch.long)
    rk = torch.as_tensor(rec // nx, dtype=torch.long)
    isrc, ksrc = src_cell
    srcz = torch.as_tensor(np.asarray(srcz, dtype=np.float64))
    ring = torch.ones_like(e11)
    ring[0, :] = 0.0
    ring[-1, :] = 0.0
    ring[:, 0] = 0.0
    ring[:, -1] = 0.0
    H = (slice(0, nx - 1), slice(0, nz - 1))    # 1-based i, j = 1..n-1
    E = (slice(1, nx), slice(1, nz))            # 1-based i, j = 2..n

    def put(a, c, val):
        out = a.clone()
        out[c] = val
        return out

    out = []
    for it in range(nt):
        c = H
        dEx_dz = (Ex[0:nx - 1, 1:nz] - Ex[c]) / dz
        dEz_dx = (Ez[1:nx, 0:nz - 1] - Ez[c]) / dx
        n0 = bc[c] * m0[c] + ac[c] * dEx_dz
        n1 = bch[c] * m1[c] + ach[c] * dEz_dx
        m0, m1 = put(m0, c, n0), put(m1, c, n1)
        dEz_dx = dEz_dx / kaph[c] + n1
        dEx_dz = dEx_dz / kap[c] + n0
        Hy = put(Hy, c, 1.0 * Hy[c] + dbHy * (dEz_dx - dEx_dz))
        c = E
        dHy_dz = (Hy[c] - Hy[1:nx, 0:nz - 1]) / dz
        dHy_dx = (Hy[c] - Hy[0:nx - 1, 1:nz]) / dx
        n2 = bch[c] * m2[c] + ach[c] * dHy_dx
        n3 = bc[c] * m3[c] + ac[c] * dHy_dz
        m2, m3 = put(m2, c, n2), put(m3, c, n3)
        dHy_dz = dHy_dz / kap[c] + n3
        dHy_dx = dHy_dx / kaph[c] + n2
        Exo, Ezo = Ex, Ez
        nEz = Ezo[c] + (-aEz[c] * dHy_dz + bEz[c] * dHy_dx - dEz[c] * Exo[c] - eEz[c] * Ezo[c]) * dt
        nEx = Exo[c] + (-aEx[c] * dHy_dz + bEx[c] * dHy_dx - dEx[c] * Exo[c] - eEx[c] * Ezo[c]) * dt
        Ez, Ex = put(Ezo, c, nEz), put(Exo, c, nEx)
        Ez = Ez.clone()
        Ez[isrc, ksrc] = Ez[isrc, ksrc] + srcz[it] * dt / e33[isrc, ksrc]
        Ex, Ez, Hy = Ex * ring, Ez * ring, Hy * ring
        out.append(torch.stack([Ex[ri, rk], Ez[ri, rk]]))
    return torch.stack(out)


def em2_misfit_and_gradient(problem, shots, observed):
    """FP64 L and dL/d{e11, e13, e33, s11, s13, s33} ((nx, nz) numpy arrays)
    for an electromag2 Problem and the shot list the GPU adjoint takes."""
    m = {k: torch.tensor(np.asarray(v, dtype=np.float64), requires_grad=k in EM_KEYS)
         for k, v in problem.model.items()}
    rec = np.asarray(problem.receivers, dtype=np.int64)
    loss = torch.zeros((), dtype=torch.float64)
    for s, shot in enumerate(shots):
        tr = em2_forward_traces(m, problem.dx, problem.dz, problem.dt, problem.time_steps,
                                (shot.xind + problem.cpml - 1, shot.zind + problem.cpml - 1), shot.srcz, rec)
        obs = torch.as_tensor(np.asarray(observed[s], dtype=np.float64).reshape(tr.shape))
        loss = loss + 0.5 * ((tr - obs) ** 2).sum()
    loss.backward()
    return float(loss.detach()), {k: m[k].grad.numpy().copy() for k in EM_KEYS}
