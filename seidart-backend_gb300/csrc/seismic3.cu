// seismic3.cu -- 3D anisotropic elastic CPML-FDTD (21 C_ij),
// src/fortran/cpmlfdtd.f08:1747-2277.
//
//   s3_stress   : the four stress loops (:1761-1992) in one pass; each cell
//                 evaluates the loops whose bounds contain it.
//   s3_velocity : vx, vy, vz (:2014-2127), force source (:2214-2219),
//                 Dirichlet faces (:2226-2248), velocity and stress max-norms
//                 (:2255-2258).
// This file is the reference-order implementation used by the FP64 drop-in
// path (one thread per cell, neighbours through L1/L2).  The FP32 fast path
// has its own z-marching kernels in seismic3_fast.cu.
#include "common.cuh"
#include "kernels.h"

namespace {
constexpr int BX = 32, BY = 4, BZ = 2;

#define IX(fi, fj, fk) \
    ((size_t)((fi) - 1) + (size_t)nx * ((size_t)((fj) - 1) + (size_t)ny * (size_t)((fk) - 1)))

#if SD_EXACT
#define D4(f, p1, p0, p2, m1, h) ((27.0 * ((f)[p1] - (f)[p0]) - ((f)[p2] - (f)[m1])) / (h))
#define KAP(d, k, m) ((d) / (k) + (m))
#else
#define D4(f, p1, p0, p2, m1, h) ((27.0f * ((f)[p1] - (f)[p0]) - ((f)[p2] - (f)[m1])) * (h))
#define KAP(d, k, m) ((d) * (k) + (m))
#endif

template <int L>
__device__ __forceinline__ void stress_loop(const S3Args<real>& a, int i, int j, int k, size_t c, bool pml) {
    const int nx = a.nx, ny = a.ny;
    // stencil direction per axis (forward = "half grid") and CPML coefficient set
    constexpr bool xf = (L == 1 || L == 4), yf = (L == 2 || L == 4), zf = (L >= 3);
    constexpr bool xh = (L == 1 || L == 4), yh = (L != 1 && L != 3), zh = (L != 1);
#if SD_EXACT
    const real hx = 24.0 * a.dx, hy = 24.0 * a.dy, hz = 24.0 * a.dz;
#else
    const real hx = 1.0f / (24.0f * a.dx), hy = 1.0f / (24.0f * a.dy), hz = 1.0f / (24.0f * a.dz);
#endif
    real g[3][3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const real* __restrict__ v = a.f[q];
        g[q][0] = xf ? D4(v, IX(i + 1, j, k), c, IX(i + 2, j, k), IX(i - 1, j, k), hx)
                     : D4(v, c, IX(i - 1, j, k), IX(i + 1, j, k), IX(i - 2, j, k), hx);
        g[q][1] = yf ? D4(v, IX(i, j + 1, k), c, IX(i, j + 2, k), IX(i, j - 1, k), hy)
                     : D4(v, c, IX(i, j - 1, k), IX(i, j + 1, k), IX(i, j - 2, k), hy);
        g[q][2] = zf ? D4(v, IX(i, j, k + 1), c, IX(i, j, k + 2), IX(i, j, k - 1), hz)
                     : D4(v, c, IX(i, j, k - 1), IX(i, j, k + 1), IX(i, j, k - 2), hz);
    }
    if (pml) {
        const real bx = a.cpml[xh ? 5 : 4][c], ax = a.cpml[xh ? 3 : 2][c], kx = a.cpml[xh ? 1 : 0][c];
        const real by = a.cpml[yh ? 5 : 4][c], ay = a.cpml[yh ? 3 : 2][c], ky = a.cpml[yh ? 1 : 0][c];
        const real bz = a.cpml[zh ? 5 : 4][c], az = a.cpml[zh ? 3 : 2][c], kz = a.cpml[zh ? 1 : 0][c];
        real* const* M = a.mem + 9 * (L - 1);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            real m;
            m = bx * M[3 * q][c] + ax * g[q][0]; M[3 * q][c] = m; g[q][0] = KAP(g[q][0], kx, m);
            m = by * M[3 * q + 1][c] + ay * g[q][1]; M[3 * q + 1][c] = m; g[q][1] = KAP(g[q][1], ky, m);
            m = bz * M[3 * q + 2][c] + az * g[q][2]; M[3 * q + 2][c] = m;
            // reference quirk (cpmlfdtd.f08:1855-1866): loop 2 updates
            // memory_dvx_dz2 but sigmaxy uses the raw dvx_dz
            if (!(L == 2 && q == 0)) g[q][2] = KAP(g[q][2], kz, m);
        }
    }
    const real dvx_dx = g[0][0], dvx_dy = g[0][1], dvx_dz = g[0][2];
    const real dvy_dx = g[1][0], dvy_dy = g[1][1], dvy_dz = g[1][2];
    const real dvz_dx = g[2][0], dvz_dy = g[2][1], dvz_dz = g[2][2];
    const real dt = a.dt;
    auto upd = [&](real* s, int c1, int c2, int c3, int c4, int c5, int c6, const real* gm) {
        const real acc = a.C[c1][c] * dvx_dx + a.C[c2][c] * dvy_dy + a.C[c3][c] * dvz_dz +
                         a.C[c4][c] * (dvy_dz + dvz_dy) + a.C[c5][c] * (dvx_dz + dvz_dx) +
                         a.C[c6][c] * (dvy_dx + dvx_dy);
#if SD_EXACT
        s[c] = (s[c] + acc * dt) / (1.0 + gm[c] * dt);
#else
        s[c] = (s[c] + acc * dt) * gm[c];
#endif
    };
    if (L == 1) {
        upd(a.f[3], 0, 1, 2, 3, 4, 5, a.g[0]);
        upd(a.f[6], 1, 6, 7, 8, 9, 10, a.g[1]);
        upd(a.f[8], 2, 7, 11, 12, 13, 14, a.g[2]);
    } else if (L == 2) {
        upd(a.f[4], 5, 10, 14, 17, 19, 20, a.g[3]);
    } else if (L == 3) {
        upd(a.f[5], 4, 9, 13, 16, 18, 19, a.g[5]);
    } else {
        upd(a.f[7], 3, 8, 12, 15, 16, 17, a.g[4]);
    }
}

__global__ void __launch_bounds__(BX* BY* BZ) s3_stress(S3Args<real> a) {
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    const int k = blockIdx.z * BZ + threadIdx.z + 1;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (i > nx || j > ny || k > nz) return;
    const size_t c = IX(i, j, k);
    const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.j0 && j - 1 < a.box.j1 &&
                       k - 1 >= a.box.k0 && k - 1 < a.box.k1);
    if (k >= 3 && k <= nz - 1 && j >= 3 && j <= ny - 1 && i >= 2 && i <= nx - 2) stress_loop<1>(a, i, j, k, c, pml);
    if (k >= 3 && k <= nz - 1 && j >= 2 && j <= ny - 2 && i >= 3 && i <= nx - 1) stress_loop<2>(a, i, j, k, c, pml);
    if (k >= 2 && k <= nz - 2 && j >= 3 && j <= ny - 1 && i >= 3 && i <= nx - 1) stress_loop<3>(a, i, j, k, c, pml);
    if (k >= 2 && k <= nz - 2 && j >= 2 && j <= ny - 2 && i >= 2 && i <= nx - 2) stress_loop<4>(a, i, j, k, c, pml);
}

__device__ __forceinline__ real face_div(real d, real r0, real r1, int code) {
#if SD_EXACT
    return d / scalar_mean_d(r0, r1, code);
#else
    return d * inv_mean_f(r0, r1, code);
#endif
}

__global__ void __launch_bounds__(BX* BY* BZ) s3_velocity(S3Args<real> a, StepInfo si) {
    const int it = *si.step;
    __shared__ double red[BX * BY * BZ / 32];
    __shared__ double red2[BX * BY * BZ / 32];
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    const int k = blockIdx.z * BZ + threadIdx.z + 1;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    double vn = 0.0, sn = 0.0;
    float vsq = 0.f, ssq = 0.f, w[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // FP32 build
    if (i <= nx && j <= ny && k <= nz) {
        const size_t c = IX(i, j, k);
        const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.j0 && j - 1 < a.box.j1 &&
                           k - 1 >= a.box.k0 && k - 1 < a.box.k1);
        const real *sxx = a.f[3], *sxy = a.f[4], *sxz = a.f[5], *syy = a.f[6], *syz = a.f[7], *szz = a.f[8];
        const real* rho = a.rho;
        const real dt = a.dt;
        const int code = a.density_code;
#if SD_EXACT
        const real hx = 24.0 * a.dx, hy = 24.0 * a.dy, hz = 24.0 * a.dz;
#else
        const real hx = 1.0f / (24.0f * a.dx), hy = 1.0f / (24.0f * a.dy), hz = 1.0f / (24.0f * a.dz);
#endif
        const real *kap = a.cpml[0], *kaph = a.cpml[1], *ac = a.cpml[2], *ach = a.cpml[3], *bc = a.cpml[4],
                   *bch = a.cpml[5];
        real vx = a.f[0][c], vy = a.f[1][c], vz = a.f[2][c];
        const real r0 = rho[c];
        if (k >= 3 && k <= nz - 1 && j >= 3 && j <= ny - 1 && i >= 3 && i <= nx - 1) {
#if SD_EXACT
            real d1 = (27.0 * sxx[c] - 27.0 * sxx[IX(i - 1, j, k)] + sxx[IX(i - 2, j, k)]) / hx;
            real d2 = (27.0 * sxy[c] - 27.0 * sxy[IX(i, j - 1, k)] + sxy[IX(i, j - 2, k)]) / hy;
            real d3 = (27.0 * sxz[c] - 27.0 * sxz[IX(i, j, k - 1)] + sxz[IX(i, j, k - 2)]) / hz;
#else
            real d1 = (27.0f * (sxx[c] - sxx[IX(i - 1, j, k)]) + sxx[IX(i - 2, j, k)]) * hx;
            real d2 = (27.0f * (sxy[c] - sxy[IX(i, j - 1, k)]) + sxy[IX(i, j - 2, k)]) * hy;
            real d3 = (27.0f * (sxz[c] - sxz[IX(i, j, k - 1)]) + sxz[IX(i, j, k - 2)]) * hz;
#endif
            if (pml) {
                real m;
                m = bch[c] * a.mem[36][c] + ach[c] * d1; a.mem[36][c] = m; d1 = KAP(d1, kaph[c], m);
                m = bch[c] * a.mem[40][c] + ach[c] * d2; a.mem[40][c] = m; d2 = KAP(d2, kaph[c], m);
                m = bch[c] * a.mem[42][c] + ach[c] * d3; a.mem[42][c] = m; d3 = KAP(d3, kaph[c], m);
            }
            vx = vx + (face_div(d1, r0, rho[IX(i - 1, j, k)], code) + face_div(d2, r0, r0, code) +
                       face_div(d3, r0, rho[IX(i, j, k - 1)], code)) * dt;
        }
        if (k >= 3 && k <= nz - 1 && j >= 2 && j <= ny - 2 && i >= 2 && i <= nx - 2) {
#if SD_EXACT
            real d1 = (-27.0 * sxy[c] + 27.0 * sxy[IX(i + 1, j, k)] - sxy[IX(i + 2, j, k)]) / hx;
            real d2 = (-27.0 * syy[c] + 27.0 * syy[IX(i, j + 1, k)] - syy[IX(i, j + 2, k)]) / hy;
            real d3 = (27.0 * syz[c] - 27.0 * syz[IX(i, j, k - 1)] + syz[IX(i, j, k - 2)]) / hz;
#else
            real d1 = (27.0f * (sxy[IX(i + 1, j, k)] - sxy[c]) - sxy[IX(i + 2, j, k)]) * hx;
            real d2 = (27.0f * (syy[IX(i, j + 1, k)] - syy[c]) - syy[IX(i, j + 2, k)]) * hy;
            real d3 = (27.0f * (syz[c] - syz[IX(i, j, k - 1)]) + syz[IX(i, j, k - 2)]) * hz;
#endif
            if (pml) {
                real m;
                m = bch[c] * a.mem[39][c] + ach[c] * d1; a.mem[39][c] = m; d1 = KAP(d1, kaph[c], m);
                m = bch[c] * a.mem[37][c] + ach[c] * d2; a.mem[37][c] = m; d2 = KAP(d2, kaph[c], m);
                m = bc[c] * a.mem[44][c] + ac[c] * d3; a.mem[44][c] = m; d3 = KAP(d3, kap[c], m);
            }
            vy = vy + (face_div(d1, r0, rho[IX(i + 1, j, k)], code) + face_div(d2, r0, r0, code) +
                       face_div(d3, r0, rho[IX(i, j, k - 1)], code)) * dt;
        }
        if (k >= 2 && k <= nz - 2 && j >= 3 && j <= ny - 1 && i >= 2 && i <= nx - 2) {
#if SD_EXACT
            real d1 = (-27.0 * sxz[c] + 27.0 * sxz[IX(i + 1, j, k)] - sxz[IX(i + 2, j, k)]) / hx;
            real d2 = (27.0 * syz[c] - 27.0 * syz[IX(i, j - 1, k)] + syz[IX(i, j - 2, k)]) / hy;
            real d3 = (-27.0 * szz[c] + 27.0 * szz[IX(i, j, k + 1)] - szz[IX(i, j, k + 2)]) / hz;
#else
            real d1 = (27.0f * (sxz[IX(i + 1, j, k)] - sxz[c]) - sxz[IX(i + 2, j, k)]) * hx;
            real d2 = (27.0f * (syz[c] - syz[IX(i, j - 1, k)]) + syz[IX(i, j - 2, k)]) * hy;
            real d3 = (27.0f * (szz[IX(i, j, k + 1)] - szz[c]) - szz[IX(i, j, k + 2)]) * hz;
#endif
            if (pml) {
                real m;
                m = bch[c] * a.mem[41][c] + ach[c] * d1; a.mem[41][c] = m; d1 = KAP(d1, kaph[c], m);
                m = bc[c] * a.mem[43][c] + ac[c] * d2; a.mem[43][c] = m; d2 = KAP(d2, kap[c], m);
                m = bch[c] * a.mem[38][c] + ach[c] * d3; a.mem[38][c] = m; d3 = KAP(d3, kaph[c], m);
            }
            vz = vz + (face_div(d1, r0, rho[IX(i + 1, j, k)], code) + face_div(d2, r0, r0, code) +
                       face_div(d3, r0, rho[IX(i, j, k + 1)], code)) * dt;
        }
        // force source, cpmlfdtd.f08:2214-2219 (with dt); densities per the reference
        const int is = a.isrc + 1, js = a.jsrc + 1, ks = a.ksrc + 1;
#define SRCDIV(x, r) ((x) / (r))
        if (a.src[0] && i == is + 1 && j == js && k == ks) vx = vx + SRCDIV((real)a.src[0][it - 1] * dt, rho[IX(is + 1, js, ks)]);
        if (a.src[1] && i == is && j == js + 1 && k == ks) vy = vy + SRCDIV((real)a.src[1][it - 1] * dt, rho[IX(is, js, ks)]);
        if (a.src[2] && i == is && j == js && k == ks + 1) vz = vz + SRCDIV((real)a.src[2][it - 1] * dt, rho[IX(is, js, ks + 1)]);
#undef SRCDIV
        if (i == 1 || i == nx || j == 1 || j == ny || k == 1 || k == nz) { vx = 0; vy = 0; vz = 0; }
        a.f[0][c] = vx;
        a.f[1][c] = vy;
        a.f[2][c] = vz;
        // stress norm: cells that a stress source touches afterwards are
        // handled by s3_stress_source
        const bool src_cell = a.stress_src && ((i == is && j == js && k == ks) || (i == is + 1 && j == js + 1 && k == ks) ||
                                               (i == is + 1 && j == js && k == ks + 1) || (i == is && j == js + 1 && k == ks + 1));
#if !SD_F32
        vn = sqrt((double)vx * vx + (double)vy * vy + (double)vz * vz);
        if (!src_cell) {
            const double s1 = sxx[c], s2 = syy[c], s3 = szz[c], s4 = sxy[c], s5 = syz[c], s6 = sxz[c];
            sn = sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6));
        }
#else
        w[0] = vx; w[1] = vy; w[2] = vz;
        vsq = vx * vx + vy * vy + vz * vz;
        if (!src_cell) {
            w[3] = sxx[c]; w[4] = syy[c]; w[5] = szz[c]; w[6] = sxy[c]; w[7] = syz[c]; w[8] = sxz[c];
            ssq = w[3] * w[3] + w[4] * w[4] + w[5] * w[5] + 2.0f * (w[6] * w[6] + w[7] * w[7] + w[8] * w[8]);
        }
#endif
        // plane-wave face cells: their norms are taken after the injection
        if (a.pw.on && pw_cell(a.pw, i - 1, j - 1, k - 1)) {
            vn = 0.0; sn = 0.0; vsq = 0.f; ssq = 0.f;
            for (float& x : w) x = 0.f;
        }
    }
#if !SD_F32
    vn = block_max<BX * BY * BZ / 32>(vn, red);
    sn = block_max<BX * BY * BZ / 32>(sn, red2);
#else
    __shared__ float redf[BX * BY * BZ / 32];
    vn = block_norm_f32<BX * BY * BZ / 32>(
        vsq, [&] { return sqrt((double)w[0] * w[0] + (double)w[1] * w[1] + (double)w[2] * w[2]); }, redf, red);
    __syncthreads();
    sn = block_norm_f32<BX * BY * BZ / 32>(
        ssq,
        [&] {
            const double s1 = w[3], s2 = w[4], s3 = w[5], s4 = w[6], s5 = w[7], s6 = w[8];
            return sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6));
        },
        redf, red2);
#endif
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        atomic_max_nonneg(&a.norms[it - 1], vn);
        atomic_max_nonneg(&a.norms[a.nt + it - 1], sn);
    }
}

// stress source (cpmlfdtd.f08:2210-2215), then the stress norm of the cells it touched
__global__ void s3_stress_source(S3Args<real> a, StepInfo si) {
    const int it = *si.step;
    const int nx = a.nx, ny = a.ny;
    const int is = a.isrc + 1, js = a.jsrc + 1, ks = a.ksrc + 1;
    const real* rho = a.rho;
    auto add = [&](real* f, size_t c, const double* s, size_t rc) {
        if (s) f[c] = f[c] + (real)s[it - 1] / rho[rc];
    };
    add(a.f[3], IX(is, js, ks), a.src[3], IX(is, js, ks));
    add(a.f[4], IX(is + 1, js + 1, ks), a.src[4], IX(is + 1, js + 1, ks));
    add(a.f[5], IX(is + 1, js, ks + 1), a.src[5], IX(is + 1, js, ks));
    add(a.f[6], IX(is, js, ks), a.src[6], IX(is, js, ks));
    add(a.f[7], IX(is, js + 1, ks + 1), a.src[7], IX(is, js, ks + 1));
    add(a.f[8], IX(is, js, ks), a.src[8], IX(is, js, ks));
    const size_t cells[4] = {IX(is, js, ks), IX(is + 1, js + 1, ks), IX(is + 1, js, ks + 1), IX(is, js + 1, ks + 1)};
    double sn = 0.0;
    for (int q = 0; q < 4; ++q) {
        const size_t c = cells[q];
        const double s1 = a.f[3][c], s2 = a.f[6][c], s3 = a.f[8][c], s4 = a.f[4][c], s5 = a.f[7][c], s6 = a.f[5][c];
        sn = nanmax(sn, sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6)));
    }
    atomic_max_nonneg(&a.norms[a.nt + it - 1], sn);
}

// Receiver gather (after the Dirichlet ring, like the reference's per-step
// snapshot) and advance of the device step counter; always the last
// kernel of a step.
__global__ void s3_epilogue(S3Args<real> a, StepInfo s) {
    const int it = *s.step;
    for (int r = threadIdx.x; r < s.nrec; r += blockDim.x) {
        const size_t base = (size_t)(it - 1) * 3 * s.nrec;
        a.traces[base + r] = a.f[0][s.rec[r]];
        a.traces[base + s.nrec + r] = a.f[1][s.rec[r]];
        a.traces[base + 2 * (size_t)s.nrec + r] = a.f[2][s.rec[r]];
    }
    __syncthreads();
    if (threadIdx.x == 0) *s.step = it + 1;
}
}  // namespace

void SD_NAME(launch_seismic3)(const S3Args<real>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h) {
    const dim3 blk(BX, BY, BZ), grd((a.nx + BX - 1) / BX, (a.ny + BY - 1) / BY, (a.nz + BZ - 1) / BZ);
    s3_stress<<<grd, blk, 0, st>>>(a);
    if (h) h->fn(h->ctx, 0, "s3_stress");
    s3_velocity<<<grd, blk, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 1, "s3_velocity");
    if (a.stress_src) {
        s3_stress_source<<<1, 1, 0, st>>>(a, s);
        if (h) h->fn(h->ctx, 2, "s3_stress_source");
    }
    if (a.pw.on) pw_seismic3<real>(a, s, st);
    s3_epilogue<<<1, 256, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 3, "s3_epilogue");
}
