"""Second, independent restatement of the reference time loops in numpy.

TEST INFRASTRUCTURE ONLY.  Written directly from src/fortran/cpmlfdtd.f08 as
whole-array slice expressions (the C restatement in oracle.c loops cell by
cell), so a transcription slip in either one shows up when the two disagree.
Both evaluate every expression left to right in IEEE double with no FMA, so
they must agree bit for bit.  Small grids only.

Index convention: R(a, b) is the 0-based slice of the reference's 1-based
inclusive range a..b; R(a, b, s) shifts it by s (the stencil offset).
"""
from __future__ import annotations

import numpy as np

EPS0 = 8.85418782e-12
MU0 = 4.0 * 3.141592653589793238462643 * 1.0e-7


def R(a, b, s=0):
    return slice(a - 1 + s, b + s)


def scalar_mean(a, b, code):
    if code == 1:
        return 2.0 * a * b / (a + b)
    if code == 2:
        return np.sqrt(a * b)
    if code == 3:
        return 0.5 * (a + b)
    return a + 0.0 * b


class _S:
    """State bag."""


def seismic2(p, nsteps):
    """cpmlfdtd.f08:311-576 on a Problem; returns fields, memories, traces, norms."""
    m = {k: np.asarray(v) for k, v in p.model.items()}
    nx, nz, dx, dz, dt = p.nx, p.nz, p.dx, p.dz, p.dt
    code = p.density_code()
    f = p.field_list()
    vx, vz, sxx, szz, sxz = f
    M = [np.zeros((nx, nz), order="F") for _ in range(12)]
    (mdvx_dx1, mdvx_dz1, mdvz_dx1, mdvz_dz1, mdvx_dx2, mdvx_dz2, mdvz_dx2, mdvz_dz2,
     mdsxx_dx, mdszz_dz, mdsxz_dx, mdsxz_dz) = M
    k, kh, a, ah, b, bh = (m[n] for n in ("kappa", "kappa_half", "acoef", "acoef_half", "bcoef", "bcoef_half"))
    src = {n: p.src.get(n) for n in ("x", "z", "xx", "xz", "zz")}
    isrc, jsrc = p.xind + p.cpml - 1, p.zind + p.cpml - 1
    rec = p.receiver_array()
    traces, norms = [], []
    for step in range(nsteps):
        it = step + 1
        # stress normal j = 3..nz-1, i = 2..nx-2
        I, J = R(2, nx - 2), R(3, nz - 1)
        c = (I, J)
        dvx_dx = (27.0 * (vx[R(2, nx - 2, 1), J] - vx[c]) - (vx[R(2, nx - 2, 2), J] - vx[R(2, nx - 2, -1), J])) / (24.0 * dx)
        dvz_dz = (27.0 * (vz[c] - vz[I, R(3, nz - 1, -1)]) - (vz[I, R(3, nz - 1, 1)] - vz[I, R(3, nz - 1, -2)])) / (24.0 * dz)
        dvz_dx = (27.0 * (vz[R(2, nx - 2, 1), J] - vz[c]) - (vz[R(2, nx - 2, 2), J] - vz[R(2, nx - 2, -1), J])) / (24.0 * dx)
        dvx_dz = (27.0 * (vx[c] - vx[I, R(3, nz - 1, -1)]) - (vx[I, R(3, nz - 1, 1)] - vx[I, R(3, nz - 1, -2)])) / (24.0 * dz)
        mdvx_dx1[c] = bh[c] * mdvx_dx1[c] + ah[c] * dvx_dx
        mdvx_dz1[c] = bh[c] * mdvx_dz1[c] + ah[c] * dvx_dz
        mdvz_dz1[c] = b[c] * mdvz_dz1[c] + a[c] * dvz_dz
        mdvz_dx1[c] = b[c] * mdvz_dx1[c] + a[c] * dvz_dx
        dvx_dx = dvx_dx / kh[c] + mdvx_dx1[c]
        dvx_dz = dvx_dz / kh[c] + mdvx_dz1[c]
        dvz_dz = dvz_dz / k[c] + mdvz_dz1[c]
        dvz_dx = dvz_dx / k[c] + mdvz_dx1[c]
        sxx[c] = (sxx[c] + (m["c11"][c] * dvx_dx + m["c13"][c] * dvz_dz + m["c15"][c] * (dvz_dx + dvx_dz)) * dt) / (1.0 + m["gamma_x"][c] * dt)
        szz[c] = (szz[c] + (m["c13"][c] * dvx_dx + m["c33"][c] * dvz_dz + m["c35"][c] * (dvz_dx + dvx_dz)) * dt) / (1.0 + m["gamma_z"][c] * dt)
        # stress shear j = 2..nz-2, i = 3..nx-1
        I, J = R(3, nx - 1), R(2, nz - 2)
        c = (I, J)
        dvx_dx = (27.0 * (vx[c] - vx[R(3, nx - 1, -1), J]) - (vx[R(3, nx - 1, 1), J] - vx[R(3, nx - 1, -2), J])) / (24.0 * dx)
        dvz_dz = (27.0 * (vz[I, R(2, nz - 2, 1)] - vz[c]) - (vz[I, R(2, nz - 2, 2)] - vz[I, R(2, nz - 2, -1)])) / (24.0 * dz)
        dvz_dx = (27.0 * (vz[c] - vz[R(3, nx - 1, -1), J]) - (vz[R(3, nx - 1, 1), J] - vz[R(3, nx - 1, -2), J])) / (24.0 * dx)
        dvx_dz = (27.0 * (vx[I, R(2, nz - 2, 1)] - vx[c]) - (vx[I, R(2, nz - 2, 2)] - vx[I, R(2, nz - 2, -1)])) / (24.0 * dz)
        mdvx_dx2[c] = bh[c] * mdvx_dx2[c] + ah[c] * dvx_dx
        mdvx_dz2[c] = bh[c] * mdvx_dz2[c] + ah[c] * dvx_dz
        mdvz_dz2[c] = bh[c] * mdvz_dz2[c] + ah[c] * dvz_dz
        mdvz_dx2[c] = bh[c] * mdvz_dx2[c] + ah[c] * dvz_dx
        dvx_dx = dvx_dx / kh[c] + mdvx_dx2[c]
        dvx_dz = dvx_dz / kh[c] + mdvx_dz2[c]
        dvz_dz = dvz_dz / kh[c] + mdvz_dz2[c]
        dvz_dx = dvz_dx / kh[c] + mdvz_dx2[c]
        sxz[c] = (sxz[c] + (m["c15"][c] * dvx_dx + m["c35"][c] * dvz_dz + m["c55"][c] * (dvz_dx + dvx_dz)) * dt) / (1.0 + m["gamma_xz"][c] * dt)
        # vx j = 3..nz-1, i = 3..nx-1
        I, J = R(3, nx - 1), R(3, nz - 1)
        c = (I, J)
        rho = m["rho"]
        rhoxx = scalar_mean(rho[c], rho[R(3, nx - 1, -1), J], code)
        rhozx = scalar_mean(rho[c], rho[I, R(3, nz - 1, -1)], code)
        d1 = (27.0 * sxx[c] - 27.0 * sxx[R(3, nx - 1, -1), J] + sxx[R(3, nx - 1, -2), J]) / (24.0 * dx)
        d2 = (27.0 * sxz[c] - 27.0 * sxz[I, R(3, nz - 1, -1)] + sxz[I, R(3, nz - 1, -2)]) / (24.0 * dz)
        mdsxx_dx[c] = b[c] * mdsxx_dx[c] + a[c] * d1
        mdsxz_dz[c] = b[c] * mdsxz_dz[c] + a[c] * d2
        d1 = d1 / k[c] + mdsxx_dx[c]
        d2 = d2 / k[c] + mdsxz_dz[c]
        vx[c] = vx[c] + dt * (d1 / rhoxx + d2 / rhozx)
        # vz j = 2..nz-2, i = 2..nx-2
        I, J = R(2, nx - 2), R(2, nz - 2)
        c = (I, J)
        rhoxz = scalar_mean(rho[c], rho[R(2, nx - 2, 1), J], code)
        rhozz = scalar_mean(rho[c], rho[I, R(2, nz - 2, 1)], code)
        d1 = (-27.0 * sxz[c] + 27.0 * sxz[R(2, nx - 2, 1), J] - sxz[R(2, nx - 2, 2), J]) / (24.0 * dx)
        d2 = (-27.0 * szz[c] + 27.0 * szz[I, R(2, nz - 2, 1)] - szz[I, R(2, nz - 2, 2)]) / (24.0 * dz)
        mdsxz_dx[c] = bh[c] * mdsxz_dx[c] + ah[c] * d1
        mdszz_dz[c] = bh[c] * mdszz_dz[c] + ah[c] * d2
        d1 = d1 / kh[c] + mdsxz_dx[c]
        d2 = d2 / kh[c] + mdszz_dz[c]
        vz[c] = vz[c] + dt * (d1 / rhoxz + d2 / rhozz)
        # point source (cpmlfdtd.f08:519-523)
        s = lambda n: 0.0 if src[n] is None else src[n][it - 1]
        sxx[isrc, jsrc] = sxx[isrc, jsrc] + s("xx") / rho[isrc, jsrc]
        sxz[isrc + 1, jsrc + 1] = sxz[isrc + 1, jsrc + 1] + s("xz") / rho[isrc + 1, jsrc + 1]
        szz[isrc, jsrc] = szz[isrc, jsrc] + s("zz") / rho[isrc, jsrc]
        vx[isrc, jsrc] = vx[isrc, jsrc] + s("x") / rho[isrc, jsrc]
        vz[isrc, jsrc] = vz[isrc, jsrc] + s("z") / rho[isrc, jsrc]
        for v in (vx, vz):
            v[0, :] = 0.0; v[-1, :] = 0.0; v[:, 0] = 0.0; v[:, -1] = 0.0
        norms.append(np.max(np.sqrt(vx ** 2 + vz ** 2)))
        traces.append(np.stack([vx.ravel(order="F")[rec], vz.ravel(order="F")[rec]]))
    return {"fields": f, "memory": M, "traces": np.array(traces), "norms": np.array(norms)}


def electromag2(p, nsteps):
    """cpmlfdtd.f08:2519-2748 on a Problem."""
    m = {k: np.asarray(v) for k, v in p.model.items()}
    nx, nz, dx, dz, dt = p.nx, p.nz, p.dx, p.dz, p.dt
    f = p.field_list()
    Ex, Ez, Hy = f
    M = [np.zeros((nx, nz), order="F") for _ in range(4)]
    mdEx_dz, mdEz_dx, mdHy_dx, mdHy_dz = M
    k, kh, a, ah, b, bh = (m[n] for n in ("kappa", "kappa_half", "acoef", "acoef_half", "bcoef", "bcoef_half"))
    e11, e13, e33 = m["e11"] * EPS0, m["e13"] * EPS0, m["e33"] * EPS0
    s11, s13, s33 = m["s11"], m["s13"], m["s33"]
    det = e11 * e33 - e13 * e13
    floor = 1.0e-18 * EPS0 * EPS0
    det = np.where(det <= floor, floor, det)
    aEx, bEx = e33 / det, -e13 / det
    dEx, eEx = (e33 * s11 - e13 * s13) / det, (e33 * s13 - e13 * s33) / det
    aEz, bEz = -e13 / det, e11 / det
    dEz, eEz = (e11 * s13 - e13 * s11) / det, (e11 * s33 - e13 * s13) / det
    dbHy = dt / MU0
    isrc, jsrc = p.xind + p.cpml - 1, p.zind + p.cpml - 1
    rec = p.receiver_array()
    srcx, srcz = p.src.get("x"), p.src.get("z")
    Exo, Ezo = Ex.copy(order="F"), Ez.copy(order="F")
    traces, norms = [], []
    for step in range(nsteps):
        it = step + 1
        I, J = R(1, nx - 1), R(1, nz - 1)
        c = (I, J)
        dEx_dz = (Ex[I, R(1, nz - 1, 1)] - Ex[c]) / dz
        dEz_dx = (Ez[R(1, nx - 1, 1), J] - Ez[c]) / dx
        mdEx_dz[c] = b[c] * mdEx_dz[c] + a[c] * dEx_dz
        mdEz_dx[c] = bh[c] * mdEz_dx[c] + ah[c] * dEz_dx
        dEz_dx = dEz_dx / kh[c] + mdEz_dx[c]
        dEx_dz = dEx_dz / k[c] + mdEx_dz[c]
        Hy[c] = 1.0 * Hy[c] + dbHy * (dEz_dx - dEx_dz)
        I, J = R(2, nx), R(2, nz)
        c = (I, J)
        dHy_dz = (Hy[c] - Hy[I, R(2, nz, -1)]) / dz
        dHy_dx = (Hy[c] - Hy[R(2, nx, -1), J]) / dx
        mdHy_dx[c] = bh[c] * mdHy_dx[c] + ah[c] * dHy_dx
        mdHy_dz[c] = b[c] * mdHy_dz[c] + a[c] * dHy_dz
        dHy_dz = dHy_dz / k[c] + mdHy_dz[c]
        dHy_dx = dHy_dx / kh[c] + mdHy_dx[c]
        Ez[c] = Ezo[c] + (-aEz[c] * dHy_dz + bEz[c] * dHy_dx - dEz[c] * Exo[c] - eEz[c] * Ezo[c]) * dt
        Ex[c] = Exo[c] + (-aEx[c] * dHy_dz + bEx[c] * dHy_dx - dEx[c] * Exo[c] - eEx[c] * Ezo[c]) * dt
        if srcx is not None:
            Ex[isrc, jsrc] = Ex[isrc, jsrc] + srcx[it - 1] * dt / e11[isrc, jsrc]
        if srcz is not None:
            Ez[isrc, jsrc] = Ez[isrc, jsrc] + srcz[it - 1] * dt / e33[isrc, jsrc]
        for v in (Ex, Ez, Hy):
            v[0, :] = 0.0; v[-1, :] = 0.0; v[:, 0] = 0.0; v[:, -1] = 0.0
        Exo[...] = Ex
        Ezo[...] = Ez
        norms.append(np.max(np.sqrt(Ex ** 2 + Ez ** 2)))
        traces.append(np.stack([Ex.ravel(order="F")[rec], Ez.ravel(order="F")[rec]]))
    return {"fields": f, "memory": M, "traces": np.array(traces), "norms": np.array(norms)}


def seismic3(p, nsteps):
    """cpmlfdtd.f08:1747-2277 on a Problem (all 44 rescalings, loop-2 quirk included)."""
    m = {k: np.asarray(v) for k, v in p.model.items()}
    nx, ny, nz = p.nx, p.ny, p.nz
    dx, dy, dz, dt = p.dx, p.dy, p.dz, p.dt
    code = p.density_code()
    f = p.field_list()
    vx, vy, vz, sxx, sxy, sxz, syy, syz, szz = f
    v = (vx, vy, vz)
    M = [np.zeros((nx, ny, nz), order="F") for _ in range(45)]
    K = {0: m["kappa"], 1: m["kappa_half"]}
    A = {0: m["acoef"], 1: m["acoef_half"]}
    B = {0: m["bcoef"], 1: m["bcoef_half"]}
    h = (dx, dy, dz)
    n = (nx, ny, nz)
    rec = p.receiver_array()
    is_, js, ks = p.xind + p.cpml - 1, p.yind + p.cpml - 1, p.zind + p.cpml - 1
    traces, vnorms, snorms = [], [], []

    def sl(rng, ax, s):
        out = list(rng)
        lo, hi = bounds[ax]
        out[ax] = R(lo, hi, s)
        return tuple(out)

    for step in range(nsteps):
        it = step + 1
        # (bounds lo/hi per axis as 1-based inclusive, forward flags, half flags)
        loops = [
            (((2, nx - 2), (3, ny - 1), (3, nz - 1)), (1, 0, 0), (1, 0, 0)),
            (((3, nx - 1), (2, ny - 2), (3, nz - 1)), (0, 1, 0), (0, 1, 1)),
            (((3, nx - 1), (3, ny - 1), (2, nz - 2)), (0, 0, 1), (0, 0, 1)),
            (((2, nx - 2), (2, ny - 2), (2, nz - 2)), (1, 1, 1), (1, 1, 1)),
        ]
        for L, (bounds, fwd, half) in enumerate(loops, start=1):
            c = tuple(R(lo, hi) for lo, hi in bounds)
            g = [[None] * 3 for _ in range(3)]
            for q in range(3):
                for ax in range(3):
                    f_ = v[q]
                    if fwd[ax]:
                        g[q][ax] = (27.0 * (f_[sl(c, ax, 1)] - f_[c]) - (f_[sl(c, ax, 2)] - f_[sl(c, ax, -1)])) / (24.0 * h[ax])
                    else:
                        g[q][ax] = (27.0 * (f_[c] - f_[sl(c, ax, -1)]) - (f_[sl(c, ax, 1)] - f_[sl(c, ax, -2)])) / (24.0 * h[ax])
            for q in range(3):
                for ax in range(3):
                    mm = M[9 * (L - 1) + 3 * q + ax]
                    mm[c] = B[half[ax]][c] * mm[c] + A[half[ax]][c] * g[q][ax]
                    if not (L == 2 and q == 0 and ax == 2):
                        g[q][ax] = g[q][ax] / K[half[ax]][c] + mm[c]
            dvx_dx, dvx_dy, dvx_dz = g[0]
            dvy_dx, dvy_dy, dvy_dz = g[1]
            dvz_dx, dvz_dy, dvz_dz = g[2]

            def upd(s, c1, c2, c3, c4, c5, c6, gam):
                s[c] = (s[c] + (m[c1][c] * dvx_dx + m[c2][c] * dvy_dy + m[c3][c] * dvz_dz + m[c4][c] * (dvy_dz + dvz_dy)
                                + m[c5][c] * (dvx_dz + dvz_dx) + m[c6][c] * (dvy_dx + dvx_dy)) * dt) / (1.0 + m[gam][c] * dt)
            if L == 1:
                upd(sxx, "c11", "c12", "c13", "c14", "c15", "c16", "gamma_x")
                upd(syy, "c12", "c22", "c23", "c24", "c25", "c26", "gamma_y")
                upd(szz, "c13", "c23", "c33", "c34", "c35", "c36", "gamma_z")
            elif L == 2:
                upd(sxy, "c16", "c26", "c36", "c46", "c56", "c66", "gamma_xy")
            elif L == 3:
                upd(sxz, "c15", "c25", "c35", "c45", "c55", "c56", "gamma_xz")
            else:
                upd(syz, "c14", "c24", "c34", "c44", "c45", "c46", "gamma_yz")
        rho = m["rho"]

        def vel(target, bounds_, terms):
            nonlocal bounds
            bounds = bounds_
            c = tuple(R(lo, hi) for lo, hi in bounds)
            acc = None
            for (fld, ax, fwd, half, mslot, rax, rs) in terms:
                if fwd:
                    d = (-27.0 * fld[c] + 27.0 * fld[sl(c, ax, 1)] - fld[sl(c, ax, 2)]) / (24.0 * h[ax])
                else:
                    d = (27.0 * fld[c] - 27.0 * fld[sl(c, ax, -1)] + fld[sl(c, ax, -2)]) / (24.0 * h[ax])
                mm = M[mslot]
                mm[c] = B[half][c] * mm[c] + A[half][c] * d
                d = d / K[half][c] + mm[c]
                r = scalar_mean(rho[c], rho[sl(c, rax, rs)] if rs else rho[c], code)
                acc = d / r if acc is None else acc + d / r
            target[c] = target[c] + acc * dt

        bounds = ((3, nx - 1), (3, ny - 1), (3, nz - 1))
        vel(vx, ((3, nx - 1), (3, ny - 1), (3, nz - 1)),
            [(sxx, 0, 0, 1, 36, 0, -1), (sxy, 1, 0, 1, 40, 1, 0), (sxz, 2, 0, 1, 42, 2, -1)])
        vel(vy, ((2, nx - 2), (2, ny - 2), (3, nz - 1)),
            [(sxy, 0, 1, 1, 39, 0, 1), (syy, 1, 1, 1, 37, 1, 0), (syz, 2, 0, 0, 44, 2, -1)])
        vel(vz, ((2, nx - 2), (3, ny - 1), (2, nz - 2)),
            [(sxz, 0, 1, 1, 41, 0, 1), (syz, 1, 0, 0, 43, 1, 0), (szz, 2, 1, 1, 38, 2, 1)])
        s = lambda nm: 0.0 if p.src.get(nm) is None else p.src[nm][it - 1]
        sxx[is_, js, ks] += s("xx") / rho[is_, js, ks]
        sxy[is_ + 1, js + 1, ks] += s("xy") / rho[is_ + 1, js + 1, ks]
        sxz[is_ + 1, js, ks + 1] += s("xz") / rho[is_ + 1, js, ks]
        syy[is_, js, ks] += s("yy") / rho[is_, js, ks]
        syz[is_, js + 1, ks + 1] += s("yz") / rho[is_, js, ks + 1]
        szz[is_, js, ks] += s("zz") / rho[is_, js, ks]
        vx[is_ + 1, js, ks] += s("x") * dt / rho[is_ + 1, js, ks]
        vy[is_, js + 1, ks] += s("y") * dt / rho[is_, js, ks]
        vz[is_, js, ks + 1] += s("z") * dt / rho[is_, js, ks + 1]
        for w in v:
            w[0] = 0.0; w[-1] = 0.0; w[:, 0] = 0.0; w[:, -1] = 0.0; w[:, :, 0] = 0.0; w[:, :, -1] = 0.0
        vnorms.append(np.max(np.sqrt(vx ** 2 + vy ** 2 + vz ** 2)))
        snorms.append(np.max(np.sqrt(sxx ** 2 + syy ** 2 + szz ** 2 + 2.0 * (sxy ** 2 + syz ** 2 + sxz ** 2))))
        traces.append(np.stack([w.ravel(order="F")[rec] for w in v]))
    return {"fields": f, "memory": M, "traces": np.array(traces), "norms": np.array([vnorms, snorms])}


def electromag3(p, nsteps):
    """cpmlfdtd.f08:3353-4001 on a Problem (point sources only)."""
    m = {k: np.asarray(v) for k, v in p.model.items()}
    nx, ny, nz = p.nx, p.ny, p.nz
    dx, dy, dz, dt = p.dx, p.dy, p.dz, p.dt
    f = p.field_list()
    Ex, Ey, Ez, Hx, Hy, Hz = f
    M = [np.zeros((nx, ny, nz), order="F") for _ in range(12)]
    (mdEx_dy, mdEy_dx, mdEx_dz, mdEz_dx, mdEz_dy, mdEy_dz,
     mdHz_dx, mdHx_dz, mdHz_dy, mdHy_dz, mdHx_dy, mdHy_dx) = M
    k, kh, a, ah, b, bh = (m[n] for n in ("kappa", "kappa_half", "acoef", "acoef_half", "bcoef", "bcoef_half"))
    e11, e12, e13 = m["e11"] * EPS0, m["e12"] * EPS0, m["e13"] * EPS0
    e22, e23, e33 = m["e22"] * EPS0, m["e23"] * EPS0, m["e33"] * EPS0
    s11, s12, s13, s22, s23, s33 = (m[n] for n in ("s11", "s12", "s13", "s22", "s23", "s33"))
    det = e11 * (e22 * e33 - e23 * e23) - e12 * (e12 * e33 - e23 * e13) + e13 * (e12 * e23 - e22 * e13)
    aEx = (e22 * e33 - e23 * e23) / det
    bEx = -((e12 * e33 - e23 * e13) / det)
    cEx = (e12 * e23 - e22 * e13) / det
    aEy, bEy, cEy = bEx, (e11 * e33 - e13 * e13) / det, -((e11 * e23 - e12 * e13) / det)
    aEz, bEz, cEz = cEx, cEy, (e11 * e22 - e12 * e12) / det
    dbH = dt / MU0
    I3 = (p.xind + p.cpml - 1, p.yind + p.cpml - 1, p.zind + p.cpml - 1)
    rec = p.receiver_array()
    Exo, Eyo, Ezo = (x.copy(order="F") for x in (Ex, Ey, Ez))
    traces, norms = [], []

    def sh(c, ax, s):
        return tuple(slice(q.start + s, q.stop + s) if d == ax else q for d, q in enumerate(c))

    for step in range(nsteps):
        it = step + 1
        c = (R(1, nx - 1), R(1, ny - 1), R(1, nz - 1))
        dEz_dy = (Ez[sh(c, 1, 1)] - Ez[c]) / dy
        dEy_dz = (Ey[sh(c, 2, 1)] - Ey[c]) / dz
        mdEy_dz[c] = bh[c] * mdEy_dz[c] + ah[c] * dEy_dz
        mdEz_dy[c] = bh[c] * mdEz_dy[c] + ah[c] * dEz_dy
        dEz_dy = dEz_dy / kh[c] + mdEz_dy[c]
        dEy_dz = dEy_dz / kh[c] + mdEy_dz[c]
        Hx[c] = 1.0 * Hx[c] + dbH * (dEy_dz - dEz_dy)
        dEx_dz = (Ex[sh(c, 2, 1)] - Ex[c]) / dz
        dEz_dx = (Ez[sh(c, 0, 1)] - Ez[c]) / dx
        mdEx_dz[c] = b[c] * mdEx_dz[c] + a[c] * dEx_dz
        mdEz_dx[c] = b[c] * mdEz_dx[c] + a[c] * dEz_dx
        dEx_dz = dEx_dz / k[c] + mdEx_dz[c]
        dEz_dx = dEz_dx / k[c] + mdEz_dx[c]
        Hy[c] = 1.0 * Hy[c] + dbH * (dEz_dx - dEx_dz)
        c = (R(1, nx - 1), R(1, ny - 1), R(2, nz - 1))
        dEx_dy = (Ex[sh(c, 1, 1)] - Ex[c]) / dy
        dEy_dx = (Ey[sh(c, 0, 1)] - Ey[c]) / dx
        mdEx_dy[c] = b[c] * mdEx_dy[c] + a[c] * dEx_dy
        mdEy_dx[c] = b[c] * mdEy_dx[c] + a[c] * dEy_dx
        dEx_dy = dEx_dy / k[c] + mdEx_dy[c]
        dEy_dx = dEy_dx / k[c] + mdEy_dx[c]
        Hz[c] = 1.0 * Hz[c] + dbH * (dEx_dy - dEy_dx)
        c = (R(2, nx - 1), R(2, ny - 1), R(2, nz - 1))
        dHz_dy = (Hz[c] - Hz[sh(c, 1, -1)]) / dy
        dHy_dz = (Hy[c] - Hy[sh(c, 2, -1)]) / dz
        dHz_dx = (Hz[c] - Hz[sh(c, 0, -1)]) / dx
        dHx_dz = (Hx[c] - Hx[sh(c, 2, -1)]) / dz
        dHy_dx = (Hy[c] - Hy[sh(c, 0, -1)]) / dx
        dHx_dy = (Hx[c] - Hx[sh(c, 1, -1)]) / dy
        mdHz_dy[c] = bh[c] * mdHz_dy[c] + ah[c] * dHz_dy
        mdHy_dz[c] = b[c] * mdHy_dz[c] + a[c] * dHy_dz
        mdHz_dx[c] = bh[c] * mdHz_dx[c] + ah[c] * dHz_dx
        mdHx_dz[c] = bh[c] * mdHx_dz[c] + ah[c] * dHx_dz
        mdHx_dy[c] = bh[c] * mdHx_dy[c] + ah[c] * dHx_dy
        mdHy_dx[c] = bh[c] * mdHy_dx[c] + ah[c] * dHy_dx
        dHz_dy = dHz_dy / kh[c] + mdHz_dy[c]
        dHy_dz = dHy_dz / k[c] + mdHy_dz[c]
        dHz_dx = dHz_dx / kh[c] + mdHz_dx[c]
        dHx_dz = dHx_dz / kh[c] + mdHx_dz[c]
        dHx_dy = dHx_dy / kh[c] + mdHx_dy[c]
        dHy_dx = dHy_dx / kh[c] + mdHy_dx[c]
        rx = dHz_dy - dHy_dz - (s11[c] * Exo[c] + s12[c] * Eyo[c] + s13[c] * Ezo[c])
        ry = dHx_dz - dHz_dx - (s12[c] * Exo[c] + s22[c] * Eyo[c] + s23[c] * Ezo[c])
        rz = dHy_dx - dHx_dy - (s13[c] * Exo[c] + s23[c] * Eyo[c] + s33[c] * Ezo[c])
        Ex[c] = Exo[c] + (aEx[c] * rx + bEx[c] * ry + cEx[c] * rz) * dt
        Ey[c] = Eyo[c] + (aEy[c] * rx + bEy[c] * ry + cEy[c] * rz) * dt
        Ez[c] = Ezo[c] + (aEz[c] * rx + bEz[c] * ry + cEz[c] * rz) * dt
        for fld, nm, e in ((Ex, "x", e11), (Ey, "y", e22), (Ez, "z", e33)):
            if p.src.get(nm) is not None:
                fld[I3] = fld[I3] + p.src[nm][it - 1] * dt / e[I3]
        for w in f:
            w[0] = 0.0; w[-1] = 0.0; w[:, 0] = 0.0; w[:, -1] = 0.0; w[:, :, 0] = 0.0; w[:, :, -1] = 0.0
        Exo[...] = Ex
        Eyo[...] = Ey
        Ezo[...] = Ez
        norms.append(np.max(np.sqrt(Ex ** 2 + Ey ** 2 + Ez ** 2)))
        traces.append(np.stack([w.ravel(order="F")[rec] for w in (Ex, Ey, Ez)]))
    return {"fields": f, "memory": M, "traces": np.array(traces), "norms": np.array(norms)}
