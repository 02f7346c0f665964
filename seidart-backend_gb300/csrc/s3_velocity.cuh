// s3_velocity.cuh -- the one-cell FP32 3D velocity update shared by the
// velocity kernels (seismic3_cell.cu) and the fused step kernel
// (seismic3_bulk.cu): the three velocity loops of seismic3
// (src/fortran/cpmlfdtd.f08:2014-2127), force source (:2214-2219), Dirichlet
// faces and the squared norms of the cell.  LD selects how the stresses and
// densities are read: LD_NC through the read-only path (the stresses were
// written by an earlier launch), LD_CA through the coherent L1/L2 path (the
// stresses were written in the same launch by other CTAs).
#pragma once
#include "s3_common.cuh"

namespace s3 {

enum { LD_NC = 0, LD_CA = 1 };
template <int LD>
__device__ __forceinline__ float ldv(const float* p) {
    if constexpr (LD == LD_NC) return __ldg(p);
    else return __ldca(p);
}

// One cell of the velocity half-step.  LEAN: the CTA's whole tile lies
// inside the inert interior box, at least two cells from every face and away
// from the source cells, so every update applies, no index needs clamping and
// no CPML, source or Dirichlet test is made.
// CODE: the density rule as a compile-time constant (1..4), or 0 to read
// A.density_code at run time
template <bool LEAN, int LD = LD_NC, int CODE = 0>
__device__ __forceinline__ void velocity_cell(const S3Args<float>& A, int it, int gx, int gy, int k, float& vsq,
                                              float& ssq, float (&w)[9]) {
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
    const size_t c = (size_t)gx + sy * gy + sz * k;
    long xm2 = -2, xm1 = -1, xp1 = 1, xp2 = 2;
    long ym2 = -2 * (long)sy, ym1 = -(long)sy, yp1 = (long)sy, yp2 = 2 * (long)sy;
    long zm2 = -2 * (long)sz, zm1 = -(long)sz, zp1 = (long)sz, zp2 = 2 * (long)sz;
    if (!LEAN) {
        xm2 = (long)cl(gx - 2, 0, nx - 1) - gx; xm1 = (long)cl(gx - 1, 0, nx - 1) - gx;
        xp1 = (long)cl(gx + 1, 0, nx - 1) - gx; xp2 = (long)cl(gx + 2, 0, nx - 1) - gx;
        ym2 = ((long)cl(gy - 2, 0, ny - 1) - gy) * (long)sy; ym1 = ((long)cl(gy - 1, 0, ny - 1) - gy) * (long)sy;
        yp1 = ((long)cl(gy + 1, 0, ny - 1) - gy) * (long)sy; yp2 = ((long)cl(gy + 2, 0, ny - 1) - gy) * (long)sy;
        zm2 = ((long)cl(k - 2, 0, nz - 1) - k) * (long)sz; zm1 = ((long)cl(k - 1, 0, nz - 1) - k) * (long)sz;
        zp1 = ((long)cl(k + 1, 0, nz - 1) - k) * (long)sz; zp2 = ((long)cl(k + 2, 0, nz - 1) - k) * (long)sz;
    }
    const float *Sxx = A.f[3] + c, *Sxy = A.f[4] + c, *Sxz = A.f[5] + c, *Syy = A.f[6] + c, *Syz = A.f[7] + c,
                *Szz = A.f[8] + c, *R = A.rho + c;
    // ---- loads
    const float sxx0 = ldv<LD>(Sxx), sxxm1 = ldv<LD>(Sxx + xm1), sxxm2 = ldv<LD>(Sxx + xm2);
    const float sxy0 = ldv<LD>(Sxy), sxyp1 = ldv<LD>(Sxy + xp1), sxyp2 = ldv<LD>(Sxy + xp2);
    const float sxyym1 = ldv<LD>(Sxy + ym1), sxyym2 = ldv<LD>(Sxy + ym2);
    const float syy0 = ldv<LD>(Syy), syyp1 = ldv<LD>(Syy + yp1), syyp2 = ldv<LD>(Syy + yp2);
    const float sxz0 = ldv<LD>(Sxz), sxzp1 = ldv<LD>(Sxz + xp1), sxzp2 = ldv<LD>(Sxz + xp2);
    const float sxzzm1 = ldv<LD>(Sxz + zm1), sxzzm2 = ldv<LD>(Sxz + zm2);
    const float syz0 = ldv<LD>(Syz), syzym1 = ldv<LD>(Syz + ym1), syzym2 = ldv<LD>(Syz + ym2);
    const float syzzm1 = ldv<LD>(Syz + zm1), syzzm2 = ldv<LD>(Syz + zm2);
    const float szz0 = ldv<LD>(Szz), szzp1 = ldv<LD>(Szz + zp1), szzp2 = ldv<LD>(Szz + zp2);
    const float r0 = ldv<LD>(R), rxm = ldv<LD>(R + xm1), rxp = ldv<LD>(R + xp1), rzm = ldv<LD>(R + zm1), rzp = ldv<LD>(R + zp1);
    float vx = A.f[0][c], vy = A.f[1][c], vz = A.f[2][c];
    const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
    const float dt = A.dt;
    const int code = CODE ? CODE : A.density_code;
    const bool pml = !LEAN && !(A.box.i0 <= gx && gx < A.box.i1 && A.box.j0 <= gy && gy < A.box.j1 && A.box.k0 <= k &&
                                k < A.box.k1);
    const bool ux = LEAN || (gx >= 2 && gx <= nx - 2 && gy >= 2 && gy <= ny - 2 && k >= 2 && k <= nz - 2);
    const bool uy = LEAN || (gx >= 1 && gx <= nx - 3 && gy >= 1 && gy <= ny - 3 && k >= 2 && k <= nz - 2);
    const bool uz = LEAN || (gx >= 1 && gx <= nx - 3 && gy >= 2 && gy <= ny - 2 && k >= 1 && k <= nz - 3);
    // shell cells: the two coefficient triples and the nine memories
    // (slots 36..44: x y z derivative memories of vx, vy, vz) are all loaded
    // before the first store, so they cost one DRAM round trip, not nine
    CpmlC ph{0.f, 0.f, 0.f}, pf{0.f, 0.f, 0.f};
    float m[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (pml) {
        const CpmlPair P = cpml_pair_at(A, c, gx, gy, k);
        ph = P.h;
        pf = P.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) m[q] = A.mem[36 + q][c];
    }
    const float byy = inv_mean_f(r0, r0, code);
    if (ux) {  // vx
        float d1 = (27.0f * (sxx0 - sxxm1) + sxxm2) * hx;
        float d2 = (27.0f * (sxy0 - sxyym1) + sxyym2) * hy;
        float d3 = (27.0f * (sxz0 - sxzzm1) + sxzzm2) * hz;
        if (pml) {
            m[0] = ph.b * m[0] + ph.a * d1; d1 = d1 * ph.k + m[0];
            m[4] = ph.b * m[4] + ph.a * d2; d2 = d2 * ph.k + m[4];
            m[6] = ph.b * m[6] + ph.a * d3; d3 = d3 * ph.k + m[6];
        }
        vx = vx + (d1 * inv_mean_f(r0, rxm, code) + d2 * byy + d3 * inv_mean_f(r0, rzm, code)) * dt;
    }
    if (uy) {  // vy
        float d1 = (27.0f * (sxyp1 - sxy0) - sxyp2) * hx;
        float d2 = (27.0f * (syyp1 - syy0) - syyp2) * hy;
        float d3 = (27.0f * (syz0 - syzzm1) + syzzm2) * hz;
        if (pml) {
            m[3] = ph.b * m[3] + ph.a * d1; d1 = d1 * ph.k + m[3];
            m[1] = ph.b * m[1] + ph.a * d2; d2 = d2 * ph.k + m[1];
            m[8] = pf.b * m[8] + pf.a * d3; d3 = d3 * pf.k + m[8];
        }
        vy = vy + (d1 * inv_mean_f(r0, rxp, code) + d2 * byy + d3 * inv_mean_f(r0, rzm, code)) * dt;
    }
    if (uz) {  // vz
        float d1 = (27.0f * (sxzp1 - sxz0) - sxzp2) * hx;
        float d2 = (27.0f * (syz0 - syzym1) + syzym2) * hy;
        float d3 = (27.0f * (szzp1 - szz0) - szzp2) * hz;
        if (pml) {
            m[5] = ph.b * m[5] + ph.a * d1; d1 = d1 * ph.k + m[5];
            m[7] = pf.b * m[7] + pf.a * d2; d2 = d2 * pf.k + m[7];
            m[2] = ph.b * m[2] + ph.a * d3; d3 = d3 * ph.k + m[2];
        }
        vz = vz + (d1 * inv_mean_f(r0, rxp, code) + d2 * byy + d3 * inv_mean_f(r0, rzp, code)) * dt;
    }
    if (pml) {  // each memory written only by the update that advanced it
        if (ux) { A.mem[36][c] = m[0]; A.mem[40][c] = m[4]; A.mem[42][c] = m[6]; }
        if (uy) { A.mem[39][c] = m[3]; A.mem[37][c] = m[1]; A.mem[44][c] = m[8]; }
        if (uz) { A.mem[41][c] = m[5]; A.mem[43][c] = m[7]; A.mem[38][c] = m[2]; }
    }
    bool src_cell = false;
    if (!LEAN) {
        // force source (cpmlfdtd.f08:2214-2219)
        const int is = A.isrc, js = A.jsrc, ks = A.ksrc;
        if (gx == is + 1 && gy == js && k == ks && A.src[0]) vx = vx + (float)A.src[0][it - 1] * dt / r0;
        if (gx == is && gy == js + 1 && k == ks && A.src[1])
            vy = vy + (float)A.src[1][it - 1] * dt / A.rho[(size_t)is + sy * js + sz * ks];
        if (gx == is && gy == js && k == ks + 1 && A.src[2]) vz = vz + (float)A.src[2][it - 1] * dt / r0;
        if (gx == 0 || gx == nx - 1 || gy == 0 || gy == ny - 1 || k == 0 || k == nz - 1) { vx = 0.f; vy = 0.f; vz = 0.f; }
        src_cell = A.stress_src && ((gx == is && gy == js && k == ks) || (gx == is + 1 && gy == js + 1 && k == ks) ||
                                    (gx == is + 1 && gy == js && k == ks + 1) || (gx == is && gy == js + 1 && k == ks + 1));
    }
    __stcs(A.f[0] + c, vx);
    __stcs(A.f[1] + c, vy);
    __stcs(A.f[2] + c, vz);
    w[0] = vx; w[1] = vy; w[2] = vz;
    vsq = vx * vx + vy * vy + vz * vz;
    if (!src_cell) {
        w[3] = sxx0; w[4] = syy0; w[5] = szz0; w[6] = sxy0; w[7] = syz0; w[8] = sxz0;
        ssq = w[3] * w[3] + w[4] * w[4] + w[5] * w[5] + 2.0f * (w[6] * w[6] + w[7] * w[7] + w[8] * w[8]);
    }
    // plane-wave face cells: their norms are taken after the injection
    if (!LEAN && A.pw.on && pw_cell(A.pw, gx, gy, k)) {
        vsq = 0.f;
        ssq = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) w[q] = 0.f;
    }
}

// true when the TW x TH tile of plane k (x0.., y0..) meets a plane-wave
// injection face (such tiles take the per-cell path, which leaves face
// cells out of the norms)
__device__ __forceinline__ bool pw_tile(const PwDev& pw, int x0, int y0, int k, int tw, int th) {
    for (int f = 0; f < pw.nface; ++f) {
        const PwFace& F = pw.face[f];
        if (k >= F.lo[2] && k <= F.hi[2] && x0 <= F.hi[0] && x0 + tw - 1 >= F.lo[0] && y0 <= F.hi[1] &&
            y0 + th - 1 >= F.lo[1])
            return true;
    }
    return false;
}

// true when the whole TW x TH tile of plane k qualifies for the lean path
template <int TW = 32, int TH = 8>
__device__ __forceinline__ bool lean_tile(const S3Args<float>& A, int x0, int y0, int k, bool sources) {
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    if (!(x0 >= 2 && x0 + TW - 1 <= nx - 3 && y0 >= 2 && y0 + TH - 1 <= ny - 3 && k >= 2 && k <= nz - 3)) return false;
    if (!(x0 >= A.box.i0 && x0 + TW <= A.box.i1 && y0 >= A.box.j0 && y0 + TH <= A.box.j1 && k >= A.box.k0 &&
          k < A.box.k1))
        return false;
    if (sources) {  // the source cells sit at (is..is+1, js..js+1, ks..ks+1)
        const int is = A.isrc, js = A.jsrc, ks = A.ksrc;
        if (k >= ks && k <= ks + 1 && is + 1 >= x0 && is < x0 + TW && js + 1 >= y0 && js < y0 + TH) return false;
    }
    if (A.pw.on && pw_tile(A.pw, x0, y0, k, TW, TH)) return false;
    return true;
}

}  // namespace s3
