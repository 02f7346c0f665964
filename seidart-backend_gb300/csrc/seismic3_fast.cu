// seismic3_fast.cu -- FP32 3D elastic CPML-FDTD step with z-marching tiles.
//
// Same scheme as seismic3.cu (src/fortran/cpmlfdtd.f08:1747-2277: four stress
// loops, three velocity loops, force source, Dirichlet faces, norms), laid
// out for HBM bandwidth:
//   * each CTA owns a TX x TY column tile and marches through ZCH planes;
//   * the current plane of every stencil field sits in shared memory with a
//     2-cell x/y halo, the z neighbours of the CTA's own columns sit in a
//     register queue, so each field value comes from HBM once per step;
//   * read-once arrays (21 C_ij, gamma, CPML coefficients) stream through
//     `ld.global.cs` (evict-first) so they do not displace stencil reuse;
//   * CPML memory variables and coefficients are touched only outside the
//     inert interior box;
//   * norms reduce per CTA into one of 64 atomic slots that the epilogue
//     folds, keeping same-address atomics off the critical path.
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int TX = 32, TY = 8, ZCH = 16;
constexpr int SX = TX + 4, SY = TY + 4;  // shared tile with a 2-cell halo
constexpr int NSLOT = 64;                // norm atomic slots per step

__device__ __forceinline__ float ldcs(const float* p) { return __ldcs(p); }

struct Geo {
    int nx, ny, nz;
    size_t sxy;  // plane stride
    __device__ __forceinline__ size_t at(int x, int y, int k) const {
        return (size_t)x + (size_t)nx * (size_t)y + sxy * (size_t)k;
    }
    __device__ __forceinline__ bool in(int x, int y, int k) const {
        return x >= 0 && x < nx && y >= 0 && y < ny && k >= 0 && k < nz;
    }
};

__device__ __forceinline__ float ldz(const float* f, const Geo& g, int x, int y, int k) {
    return g.in(x, y, k) ? f[g.at(x, y, k)] : 0.0f;
}

// fill the halo ring of a shared plane (cells outside the TX x TY interior);
// the four corners are never read (no mixed derivatives)
__device__ __forceinline__ void fill_halo(float (*s)[SX], const float* f, const Geo& g, int x0, int y0, int k,
                                          int tid) {
    for (int h = tid; h < SX * SY; h += TX * TY) {
        const int hx = h % SX, hy = h / SX;
        const bool inx = hx >= 2 && hx < TX + 2, iny = hy >= 2 && hy < TY + 2;
        if (inx == iny) continue;  // interior (written from registers) or corner
        s[hy][hx] = ldz(f, g, x0 + hx - 2, y0 + hy - 2, k);
    }
}

struct CpmlC {
    float b, a, k;  // k holds 1/kappa in the FP32 build
};
__device__ __forceinline__ CpmlC cpml_at(const S3Args<float>& A, size_t c, bool half) {
    return half ? CpmlC{ldcs(A.cpml[5] + c), ldcs(A.cpml[3] + c), ldcs(A.cpml[1] + c)}
                : CpmlC{ldcs(A.cpml[4] + c), ldcs(A.cpml[2] + c), ldcs(A.cpml[0] + c)};
}
__device__ __forceinline__ float cpml_apply(float* m, size_t c, const CpmlC& p, float d) {
    const float mv = p.b * m[c] + p.a * d;
    m[c] = mv;
    return d * p.k + mv;
}

// rescale one loop's 9 derivatives through its CPML memories (shell cells only)
template <int L>
__device__ __forceinline__ void loop_cpml(const S3Args<float>& A, size_t c, float (&gx)[3], float (&gy)[3],
                                          float (&gz)[3]) {
    constexpr bool xh = (L == 1 || L == 4), yh = (L == 2 || L == 4), zh = (L != 1);
    const CpmlC px = cpml_at(A, c, xh), py = cpml_at(A, c, yh), pz = cpml_at(A, c, zh);
    float* const* M = A.mem + 9 * (L - 1);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        gx[f] = cpml_apply(M[3 * f], c, px, gx[f]);
        gy[f] = cpml_apply(M[3 * f + 1], c, py, gy[f]);
        if (L == 2 && f == 0) {
            // loop 2 advances memory_dvx_dz2 but sigma_xy uses the raw dvx_dz
            // (reference quirk, cpmlfdtd.f08:1855-1866)
            M[2][c] = pz.b * M[2][c] + pz.a * gz[0];
        } else {
            gz[f] = cpml_apply(M[3 * f + 2], c, pz, gz[f]);
        }
    }
}

// sigma <- (sigma + dt * sum C e) / (1 + gamma dt); gm holds 1/(1+gamma dt)
__device__ __forceinline__ void stress_upd(const S3Args<float>& A, size_t c, float* s, int c1, int c2, int c3,
                                           int c4, int c5, int c6, const float* gm, const float (&gx)[3],
                                           const float (&gy)[3], const float (&gz)[3]) {
    const float acc = ldcs(A.C[c1] + c) * gx[0] + ldcs(A.C[c2] + c) * gy[1] + ldcs(A.C[c3] + c) * gz[2] +
                      ldcs(A.C[c4] + c) * (gz[1] + gy[2]) + ldcs(A.C[c5] + c) * (gz[0] + gx[2]) +
                      ldcs(A.C[c6] + c) * (gx[1] + gy[0]);
    __stcs(s + c, (ldcs(s + c) + acc * A.dt) * ldcs(gm + c));
}

// ---------------------------------------------------------------- stress
__global__ void __launch_bounds__(TX* TY, 2) s3f_stress(S3Args<float> A) {
    __shared__ float sv[3][SY][SX];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int gx = x0 + tx, gy = y0 + ty;
    const Geo g{A.nx, A.ny, A.nz, (size_t)A.nx * A.ny};
    const int kb = blockIdx.z * ZCH, ke = min(kb + ZCH, A.nz);
    const bool col = gx < A.nx && gy < A.ny;
    const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    // loop membership of this column (0-based bounds of the four stress loops)
    const bool x14 = gx >= 1 && gx <= nx - 3, x23 = gx >= 2 && gx <= nx - 2;
    const bool y13 = gy >= 2 && gy <= ny - 2, y24 = gy >= 1 && gy <= ny - 3;
    const bool colbox = A.box.i0 <= gx && gx < A.box.i1 && A.box.j0 <= gy && gy < A.box.j1;

    float q[3][5];  // vx, vy, vz at planes k-2 .. k+2 of this column
#pragma unroll
    for (int f = 0; f < 3; ++f)
#pragma unroll
        for (int d = 0; d < 4; ++d) q[f][d] = col ? ldz(A.f[f], g, gx, gy, kb - 2 + d) : 0.0f;

    for (int k = kb; k < ke; ++k) {
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            q[f][4] = col ? ldz(A.f[f], g, gx, gy, k + 2) : 0.0f;
            sv[f][ty + 2][tx + 2] = q[f][2];
            fill_halo(sv[f], A.f[f], g, x0, y0, k, tid);
        }
        __syncthreads();
        const bool z12 = k >= 2 && k <= nz - 2, z34 = k >= 1 && k <= nz - 3;
        const bool L1 = col && x14 && y13 && z12, L2 = col && x23 && y24 && z12;
        const bool L3 = col && x23 && y13 && z34, L4 = col && x14 && y24 && z34;
        if (L1 || L2 || L3 || L4) {
            const size_t c = g.at(gx, gy, k);
            float fx[3], bx[3], fy[3], by[3], fz[3], bz[3];
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                const float* r = &sv[f][ty + 2][tx + 2];
                fx[f] = (27.0f * (r[1] - r[0]) - (r[2] - r[-1])) * hx;
                bx[f] = (27.0f * (r[0] - r[-1]) - (r[1] - r[-2])) * hx;
                fy[f] = (27.0f * (r[SX] - r[0]) - (r[2 * SX] - r[-SX])) * hy;
                by[f] = (27.0f * (r[0] - r[-SX]) - (r[SX] - r[-2 * SX])) * hy;
                fz[f] = (27.0f * (q[f][3] - q[f][2]) - (q[f][4] - q[f][1])) * hz;
                bz[f] = (27.0f * (q[f][2] - q[f][1]) - (q[f][3] - q[f][0])) * hz;
            }
            const bool pml = !(colbox && A.box.k0 <= k && k < A.box.k1);
            // C index: 0 c11 1 c12 2 c13 3 c14 4 c15 5 c16 6 c22 7 c23 8 c24 9 c25 10 c26
            //          11 c33 12 c34 13 c35 14 c36 15 c44 16 c45 17 c46 18 c55 19 c56 20 c66
            if (L1) {  // forward x, backward y, backward z: sigma_xx, yy, zz
                float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {bz[0], bz[1], bz[2]};
                if (pml) loop_cpml<1>(A, c, ex, ey, ez);
                stress_upd(A, c, A.f[3], 0, 1, 2, 3, 4, 5, A.g[0], ex, ey, ez);
                stress_upd(A, c, A.f[6], 1, 6, 7, 8, 9, 10, A.g[1], ex, ey, ez);
                stress_upd(A, c, A.f[8], 2, 7, 11, 12, 13, 14, A.g[2], ex, ey, ez);
            }
            if (L2) {  // backward x, forward y, backward z: sigma_xy
                float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {bz[0], bz[1], bz[2]};
                if (pml) loop_cpml<2>(A, c, ex, ey, ez);
                stress_upd(A, c, A.f[4], 5, 10, 14, 17, 19, 20, A.g[3], ex, ey, ez);
            }
            if (L3) {  // backward x, backward y, forward z: sigma_xz
                float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {fz[0], fz[1], fz[2]};
                if (pml) loop_cpml<3>(A, c, ex, ey, ez);
                stress_upd(A, c, A.f[5], 4, 9, 13, 16, 18, 19, A.g[5], ex, ey, ez);
            }
            if (L4) {  // forward x, y, z: sigma_yz
                float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {fz[0], fz[1], fz[2]};
                if (pml) loop_cpml<4>(A, c, ex, ey, ez);
                stress_upd(A, c, A.f[7], 3, 8, 12, 15, 16, 17, A.g[4], ex, ey, ez);
            }
        }
        __syncthreads();
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int d = 0; d < 4; ++d) q[f][d] = q[f][d + 1];
    }
}

// -------------------------------------------------------------- velocity
// shared planes: 0 sigma_xx, 1 sigma_xy, 2 sigma_yy, 3 sigma_xz, 4 sigma_yz, 5 rho
__global__ void __launch_bounds__(TX* TY, 2) s3f_velocity(S3Args<float> A, StepInfo si) {
    __shared__ float sp[6][SY][SX];
    __shared__ double red[2][TX * TY / 32];
    const int it = *si.step;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int gx = x0 + tx, gy = y0 + ty;
    const Geo g{A.nx, A.ny, A.nz, (size_t)A.nx * A.ny};
    const int kb = blockIdx.z * ZCH, ke = min(kb + ZCH, A.nz);
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    const bool col = gx < nx && gy < ny;
    const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
    const float dt = A.dt;
    const int code = A.density_code;
    const bool colbox = A.box.i0 <= gx && gx < A.box.i1 && A.box.j0 <= gy && gy < A.box.j1;
    // loop membership of this column
    const bool x5 = gx >= 2 && gx <= nx - 2, y5 = gy >= 2 && gy <= ny - 2;
    const bool x67 = gx >= 1 && gx <= nx - 3, y6 = gy >= 1 && gy <= ny - 3;
    const bool face_xy = gx == 0 || gx == nx - 1 || gy == 0 || gy == ny - 1;
    const int is = A.isrc, js = A.jsrc, ks = A.ksrc;
    float* const* F = A.f;
    // z queues of this column: sigma_xz, sigma_yz (k-2..k), sigma_zz (k..k+2), rho (k-1..k+1)
    float qxz[3], qyz[3], qzz[3], qr[3];
    qxz[0] = col ? ldz(F[5], g, gx, gy, kb - 2) : 0.f; qxz[1] = col ? ldz(F[5], g, gx, gy, kb - 1) : 0.f;
    qyz[0] = col ? ldz(F[7], g, gx, gy, kb - 2) : 0.f; qyz[1] = col ? ldz(F[7], g, gx, gy, kb - 1) : 0.f;
    qzz[0] = col ? ldz(F[8], g, gx, gy, kb) : 0.f; qzz[1] = col ? ldz(F[8], g, gx, gy, kb + 1) : 0.f;
    qr[0] = col ? ldz(A.rho, g, gx, gy, kb - 1) : 0.f; qr[1] = col ? ldz(A.rho, g, gx, gy, kb) : 0.f;
    double vmax = 0.0, smax = 0.0;
    float vsq = 0.f, ssq = 0.f;
    for (int k = kb; k < ke; ++k) {
        const size_t c = g.at(gx, gy, k);
        qzz[2] = col ? ldz(F[8], g, gx, gy, k + 2) : 0.f;
        qr[2] = col ? ldz(A.rho, g, gx, gy, k + 1) : 0.f;
        float sxx = 0.f, sxy = 0.f, syy = 0.f;
        if (col) {
            sxx = F[3][c]; sxy = F[4][c]; syy = F[6][c];
            qxz[2] = F[5][c]; qyz[2] = F[7][c];
        } else {
            qxz[2] = 0.f; qyz[2] = 0.f;
        }
        sp[0][ty + 2][tx + 2] = sxx;
        sp[1][ty + 2][tx + 2] = sxy;
        sp[2][ty + 2][tx + 2] = syy;
        sp[3][ty + 2][tx + 2] = qxz[2];
        sp[4][ty + 2][tx + 2] = qyz[2];
        sp[5][ty + 2][tx + 2] = qr[1];
        fill_halo(sp[0], F[3], g, x0, y0, k, tid);
        fill_halo(sp[1], F[4], g, x0, y0, k, tid);
        fill_halo(sp[2], F[6], g, x0, y0, k, tid);
        fill_halo(sp[3], F[5], g, x0, y0, k, tid);
        fill_halo(sp[4], F[7], g, x0, y0, k, tid);
        fill_halo(sp[5], A.rho, g, x0, y0, k, tid);
        __syncthreads();
        if (col) {
            const bool pml = !(colbox && A.box.k0 <= k && k < A.box.k1);
            const float r0 = qr[1];
            float vx = F[0][c], vy = F[1][c], vz = F[2][c];
            if (x5 && y5 && k >= 2 && k <= nz - 2) {  // vx, cpmlfdtd.f08:2014-2034
                const float* a = &sp[0][ty + 2][tx + 2];
                const float* b = &sp[1][ty + 2][tx + 2];
                float d1 = (27.0f * (a[0] - a[-1]) + a[-2]) * hx;
                float d2 = (27.0f * (b[0] - b[-SX]) + b[-2 * SX]) * hy;
                float d3 = (27.0f * (qxz[2] - qxz[1]) + qxz[0]) * hz;
                if (pml) {
                    const CpmlC p = cpml_at(A, c, true);
                    d1 = cpml_apply(A.mem[36], c, p, d1);
                    d2 = cpml_apply(A.mem[40], c, p, d2);
                    d3 = cpml_apply(A.mem[42], c, p, d3);
                }
                vx = vx + (d1 * inv_mean_f(r0, sp[5][ty + 2][tx + 1], code) + d2 * inv_mean_f(r0, r0, code) +
                           d3 * inv_mean_f(r0, qr[0], code)) * dt;
            }
            if (x67 && y6 && k >= 2 && k <= nz - 2) {  // vy, cpmlfdtd.f08:2055-2076
                const float* b = &sp[1][ty + 2][tx + 2];
                const float* e = &sp[2][ty + 2][tx + 2];
                float d1 = (27.0f * (b[1] - b[0]) - b[2]) * hx;
                float d2 = (27.0f * (e[SX] - e[0]) - e[2 * SX]) * hy;
                float d3 = (27.0f * (qyz[2] - qyz[1]) + qyz[0]) * hz;
                if (pml) {
                    const CpmlC ph = cpml_at(A, c, true), pf = cpml_at(A, c, false);
                    d1 = cpml_apply(A.mem[39], c, ph, d1);
                    d2 = cpml_apply(A.mem[37], c, ph, d2);
                    d3 = cpml_apply(A.mem[44], c, pf, d3);
                }
                vy = vy + (d1 * inv_mean_f(r0, sp[5][ty + 2][tx + 3], code) + d2 * inv_mean_f(r0, r0, code) +
                           d3 * inv_mean_f(r0, qr[0], code)) * dt;
            }
            if (x67 && y5 && k >= 1 && k <= nz - 3) {  // vz, cpmlfdtd.f08:2098-2120
                const float* a = &sp[3][ty + 2][tx + 2];
                const float* b = &sp[4][ty + 2][tx + 2];
                float d1 = (27.0f * (a[1] - a[0]) - a[2]) * hx;
                float d2 = (27.0f * (b[0] - b[-SX]) + b[-2 * SX]) * hy;
                float d3 = (27.0f * (qzz[1] - qzz[0]) - qzz[2]) * hz;
                if (pml) {
                    const CpmlC ph = cpml_at(A, c, true), pf = cpml_at(A, c, false);
                    d1 = cpml_apply(A.mem[41], c, ph, d1);
                    d2 = cpml_apply(A.mem[43], c, pf, d2);
                    d3 = cpml_apply(A.mem[38], c, ph, d3);
                }
                vz = vz + (d1 * inv_mean_f(r0, sp[5][ty + 2][tx + 3], code) + d2 * inv_mean_f(r0, r0, code) +
                           d3 * inv_mean_f(r0, qr[2], code)) * dt;
            }
            // force source (cpmlfdtd.f08:2214-2219), after all updates of this cell
            if (gx == is + 1 && gy == js && k == ks && A.src[0]) vx = vx + (float)A.src[0][it - 1] * dt / r0;
            if (gx == is && gy == js + 1 && k == ks && A.src[1]) vy = vy + (float)A.src[1][it - 1] * dt / ldz(A.rho, g, is, js, ks);
            if (gx == is && gy == js && k == ks + 1 && A.src[2]) vz = vz + (float)A.src[2][it - 1] * dt / r0;
            if (face_xy || k == 0 || k == nz - 1) { vx = 0.f; vy = 0.f; vz = 0.f; }
            F[0][c] = vx;
            F[1][c] = vy;
            F[2][c] = vz;
            // squared norms in FP32 (FP64 throughput on this part is a small
            // fraction of FP32); squares that would overflow FP32, or NaN,
            // take the FP64 route so the blow-up test stays exact
            const float vs = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
            if (vs < 3.0e38f) vsq = fmaxf(vsq, vs);
            else vmax = nanmax(vmax, sqrt((double)vx * vx + (double)vy * vy + (double)vz * vz));
            const bool src_cell = A.stress_src && ((gx == is && gy == js && k == ks) || (gx == is + 1 && gy == js + 1 && k == ks) ||
                                                   (gx == is + 1 && gy == js && k == ks + 1) || (gx == is && gy == js + 1 && k == ks + 1));
            if (!src_cell) {
                const float s1 = sxx, s2 = syy, s3 = qzz[0], s4 = sxy, s5 = qyz[2], s6 = qxz[2];
                const float ss = fmaf(s1, s1, fmaf(s2, s2, s3 * s3)) + 2.0f * fmaf(s4, s4, fmaf(s5, s5, s6 * s6));
                if (ss < 3.0e38f) ssq = fmaxf(ssq, ss);
                else {
                    const double d1 = s1, d2 = s2, d3 = s3, d4 = s4, d5 = s5, d6 = s6;
                    smax = nanmax(smax, sqrt(d1 * d1 + d2 * d2 + d3 * d3 + 2.0 * (d4 * d4 + d5 * d5 + d6 * d6)));
                }
            }
        }
        __syncthreads();
        qxz[0] = qxz[1]; qxz[1] = qxz[2];
        qyz[0] = qyz[1]; qyz[1] = qyz[2];
        qzz[0] = qzz[1]; qzz[1] = qzz[2];
        qr[0] = qr[1]; qr[1] = qr[2];
    }
    __shared__ float redf[2][TX * TY / 32];
    const float vq = block_maxf<TX * TY / 32>(vsq, redf[0]);
    const float sq2 = block_maxf<TX * TY / 32>(ssq, redf[1]);
    vmax = block_max<TX * TY / 32>(vmax, red[0]);  // FP64 fall-back values (normally 0)
    smax = block_max<TX * TY / 32>(smax, red[1]);
    if (tid == 0) {
        vmax = nanmax(vmax, sqrt((double)vq));
        smax = nanmax(smax, sqrt((double)sq2));
        const int slot = (blockIdx.x + 7 * blockIdx.y + 13 * blockIdx.z) % NSLOT;
        atomic_max_nonneg(A.norms_part + slot, vmax);
        atomic_max_nonneg(A.norms_part + NSLOT + slot, smax);
    }
}

// stress source (cpmlfdtd.f08:2210-2215) and the stress norm of the cells it touches
__global__ void s3f_stress_source(S3Args<float> A, StepInfo si) {
    const int it = *si.step;
    const Geo g{A.nx, A.ny, A.nz, (size_t)A.nx * A.ny};
    const int is = A.isrc, js = A.jsrc, ks = A.ksrc;
    const float* rho = A.rho;
    auto add = [&](float* f, size_t c, const double* s, size_t rc) {
        if (s) f[c] = f[c] + (float)s[it - 1] / rho[rc];
    };
    add(A.f[3], g.at(is, js, ks), A.src[3], g.at(is, js, ks));
    add(A.f[4], g.at(is + 1, js + 1, ks), A.src[4], g.at(is + 1, js + 1, ks));
    add(A.f[5], g.at(is + 1, js, ks + 1), A.src[5], g.at(is + 1, js, ks));
    add(A.f[6], g.at(is, js, ks), A.src[6], g.at(is, js, ks));
    add(A.f[7], g.at(is, js + 1, ks + 1), A.src[7], g.at(is, js, ks + 1));
    add(A.f[8], g.at(is, js, ks), A.src[8], g.at(is, js, ks));
    const size_t cells[4] = {g.at(is, js, ks), g.at(is + 1, js + 1, ks), g.at(is + 1, js, ks + 1), g.at(is, js + 1, ks + 1)};
    double sn = 0.0;
    for (int q = 0; q < 4; ++q) {
        const size_t c = cells[q];
        const double s1 = A.f[3][c], s2 = A.f[6][c], s3 = A.f[8][c], s4 = A.f[4][c], s5 = A.f[7][c], s6 = A.f[5][c];
        sn = nanmax(sn, sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6)));
    }
    atomic_max_nonneg(A.norms_part + NSLOT, sn);
}

// receivers, norm slot folding (then reset) and the step counter
__global__ void s3f_epilogue(S3Args<float> A, StepInfo s) {
    __shared__ double red[2][8];
    const int it = *s.step;
    for (int r = threadIdx.x; r < s.nrec; r += blockDim.x) {
        const size_t base = (size_t)(it - 1) * 3 * s.nrec;
        A.traces[base + r] = A.f[0][s.rec[r]];
        A.traces[base + s.nrec + r] = A.f[1][s.rec[r]];
        A.traces[base + 2 * (size_t)s.nrec + r] = A.f[2][s.rec[r]];
    }
    double v = 0.0, w = 0.0;
    if (threadIdx.x < NSLOT) {
        v = A.norms_part[threadIdx.x];
        w = A.norms_part[NSLOT + threadIdx.x];
    }
    v = block_max<8>(v, red[0]);
    w = block_max<8>(w, red[1]);
    __syncthreads();
    if (threadIdx.x < NSLOT) {
        A.norms_part[threadIdx.x] = 0.0;
        A.norms_part[NSLOT + threadIdx.x] = 0.0;
    }
    // the fused step's work ticket and plane counters start the next step at zero
    if (A.wave_ctl)
        for (int q = threadIdx.x; q < A.wave_n; q += blockDim.x) A.wave_ctl[q] = 0;
    if (threadIdx.x == 0) {
        // plane waves: the face cells' norms were written by the injection
        A.norms[it - 1] = A.pw.on ? nanmax(A.norms[it - 1], v) : v;
        A.norms[A.nt + it - 1] = A.pw.on ? nanmax(A.norms[A.nt + it - 1], w) : w;
        *s.step = it + 1;
    }
}

}  // namespace

void launch_seismic3_fast(const S3Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h,
                          const S3Maps* maps, int stress_kind, int velocity_kind) {
    const dim3 blk(TX, TY), grd((a.nx + TX - 1) / TX, (a.ny + TY - 1) / TY, (a.nz + ZCH - 1) / ZCH);
    if (a.wave_ctl && a.staged && !a.pw.on) {
        // both half-steps in one launch
        launch_seismic3_wave(a, *(const S3XMaps*)a.staged, s, st);
        if (h) h->fn(h->ctx, 0, "s3w_step");
        if (a.stress_src) {
            s3f_stress_source<<<1, 1, 0, st>>>(a, s);
            if (h) h->fn(h->ctx, 2, "s3f_stress_source");
        }
        s3f_epilogue<<<1, 256, 0, st>>>(a, s);
        if (h) h->fn(h->ctx, 3, "s3f_epilogue");
        return;
    }
    if (stress_kind == S3K_BULK && (a.packed || a.mat_ids) && a.staged) {
        launch_seismic3_staged_stress(a, *(const S3XMaps*)a.staged, st);
        if (h) h->fn(h->ctx, 0, "s3x_stress");
    } else if (stress_kind == S3K_BULK && a.packed) {
        launch_seismic3_bulk_stress(a, a.bulk_variant, st);
        if (h) h->fn(h->ctx, 0, "s3b_stress");
    } else if (stress_kind == S3K_TMA && maps) {
        launch_seismic3_tma_stress(a, *maps, st);
        if (h) h->fn(h->ctx, 0, "s3t_stress");
    } else if (stress_kind == S3K_ZMARCH) {
        s3f_stress<<<grd, blk, 0, st>>>(a);
        if (h) h->fn(h->ctx, 0, "s3f_stress");
    } else {
        launch_seismic3_cell_stress(a, st);
        if (h) h->fn(h->ctx, 0, "s3c_stress");
    }
    // plane waves need the kernels that leave face cells out of the norms:
    // the cell-pair or one-cell velocity kernel
    if (velocity_kind == S3K_CELL && a.staged_v && !a.pw.on) {
        launch_seismic3_staged_velocity(a, *(const S3XMaps*)a.staged_v, s, st);
        if (h) h->fn(h->ctx, 1, "s3x_velocity");
    } else if (velocity_kind == S3K_ZMARCH && !a.pw.on) {
        s3f_velocity<<<grd, blk, 0, st>>>(a, s);
        if (h) h->fn(h->ctx, 1, "s3f_velocity");
    } else if (a.velocity_pair) {
        launch_seismic3_pair_velocity(a, s, st);
        if (h) h->fn(h->ctx, 1, "s3p_velocity");
    } else {
        launch_seismic3_cell_velocity(a, s, st);
        if (h) h->fn(h->ctx, 1, "s3c_velocity");
    }
    if (a.stress_src) {
        s3f_stress_source<<<1, 1, 0, st>>>(a, s);
        if (h) h->fn(h->ctx, 2, "s3f_stress_source");
    }
    if (a.pw.on) {
        pw_seismic3<float>(a, s, st);  // face injection and the face cells' norms
        if (h) h->fn(h->ctx, 5, "pw_faces");
    }
    s3f_epilogue<<<1, 256, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 3, "s3f_epilogue");
}

int seismic3_fast_norm_slots() { return NSLOT; }
