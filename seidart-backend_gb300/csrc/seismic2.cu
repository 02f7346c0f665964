// seismic2.cu -- 2D anisotropic elastic (P-SV) velocity-stress CPML-FDTD.
//
// One leapfrog step = two fused half-step kernels:
//   s2_stress   : sigma_xx, sigma_zz (cpmlfdtd.f08:324-353) and sigma_xz
//                 (:362-386) with their CPML memory variables and attenuation.
//   s2_velocity : vx (:399-416), vz (:428-446), the force source (:519-523),
//                 the Dirichlet ring (:534-549), the max-norm (:552-567) and
//                 the receiver gather, all in one pass over the grid.
// A stress source (non-'ac' source types) needs its own one-thread launch
// after s2_velocity, because the reference adds it after the velocity update
// has read sigma.
//
// FP64 build: every expression keeps the reference's operation order and
// uses true divisions (compiled with --fmad=false), so each cell reproduces
// the restatement in oracle/ bit for bit.  FP32 build: the same scheme with
// precomputed reciprocals (1/kappa, 1/(1+gamma dt), 1/(24 dx)) and FMAs.
#include "common.cuh"
#include "kernels.h"

#define IX(fi, fk) ((size_t)((fi) - 1) + (size_t)a.nx * (size_t)((fk) - 1))

namespace {

constexpr int BX = 32, BY = 8;

__global__ void __launch_bounds__(BX* BY) s2_stress(S2Args<real> a) {
    const int i = blockIdx.x * BX + threadIdx.x + 1;  // Fortran indices
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    const bool normal = (j >= 3 && j <= nz - 1 && i >= 2 && i <= nx - 2);
    const bool shear = (j >= 2 && j <= nz - 2 && i >= 3 && i <= nx - 1);
    if (!normal && !shear) return;
    const size_t c = IX(i, j);
    const real* __restrict__ vx = a.f[1 - 1];
    const real* __restrict__ vz = a.f[1];
    const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.k0 && j - 1 < a.box.k1);
    const real dt = a.dt;
#if SD_EXACT
    const real hx = 24.0 * a.dx, hz = 24.0 * a.dz;
#define D4(p1, p0, p2, m1, h) ((27.0 * ((p1) - (p0)) - ((p2) - (m1))) / (h))
#define KAP(d, k, m) ((d) / (k) + (m))
#else
    const real hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
#define D4(p1, p0, p2, m1, h) ((27.0f * ((p1) - (p0)) - ((p2) - (m1))) * (h))
#define KAP(d, k, m) ((d) * (k) + (m))
#endif
    const real* __restrict__ kap = a.m[10];
    const real* __restrict__ kaph = a.m[11];
    const real* __restrict__ ac = a.m[12];
    const real* __restrict__ ach = a.m[13];
    const real* __restrict__ bc = a.m[14];
    const real* __restrict__ bch = a.m[15];
    if (normal) {
        real dvx_dx = D4(vx[IX(i + 1, j)], vx[c], vx[IX(i + 2, j)], vx[IX(i - 1, j)], hx);
        real dvz_dz = D4(vz[c], vz[IX(i, j - 1)], vz[IX(i, j + 1)], vz[IX(i, j - 2)], hz);
        real dvz_dx = D4(vz[IX(i + 1, j)], vz[c], vz[IX(i + 2, j)], vz[IX(i - 1, j)], hx);
        real dvx_dz = D4(vx[c], vx[IX(i, j - 1)], vx[IX(i, j + 1)], vx[IX(i, j - 2)], hz);
        if (pml) {
            real* m0 = a.mem[0]; real* m1 = a.mem[1]; real* m2 = a.mem[2]; real* m3 = a.mem[3];
            const real bh = bch[c], ah = ach[c], b = bc[c], aa = ac[c];
            const real M0 = bh * m0[c] + ah * dvx_dx;  // memory_dvx_dx1
            const real M1 = bh * m1[c] + ah * dvx_dz;  // memory_dvx_dz1
            const real M3 = b * m3[c] + aa * dvz_dz;   // memory_dvz_dz1
            const real M2 = b * m2[c] + aa * dvz_dx;   // memory_dvz_dx1
            m0[c] = M0; m1[c] = M1; m2[c] = M2; m3[c] = M3;
            dvx_dx = KAP(dvx_dx, kaph[c], M0);
            dvx_dz = KAP(dvx_dz, kaph[c], M1);
            dvz_dz = KAP(dvz_dz, kap[c], M3);
            dvz_dx = KAP(dvz_dx, kap[c], M2);
        }
        real* sxx = a.f[2];
        real* szz = a.f[3];
        const real c11 = a.m[0][c], c13 = a.m[1][c], c15 = a.m[2][c], c33 = a.m[3][c], c35 = a.m[4][c];
#if SD_EXACT
        sxx[c] = (sxx[c] + (c11 * dvx_dx + c13 * dvz_dz + c15 * (dvz_dx + dvx_dz)) * dt) / (1.0 + a.m[7][c] * dt);
        szz[c] = (szz[c] + (c13 * dvx_dx + c33 * dvz_dz + c35 * (dvz_dx + dvx_dz)) * dt) / (1.0 + a.m[8][c] * dt);
#else
        sxx[c] = (sxx[c] + (c11 * dvx_dx + c13 * dvz_dz + c15 * (dvz_dx + dvx_dz)) * dt) * a.m[7][c];
        szz[c] = (szz[c] + (c13 * dvx_dx + c33 * dvz_dz + c35 * (dvz_dx + dvx_dz)) * dt) * a.m[8][c];
#endif
    }
    if (shear) {
        real dvx_dx = D4(vx[c], vx[IX(i - 1, j)], vx[IX(i + 1, j)], vx[IX(i - 2, j)], hx);
        real dvz_dz = D4(vz[IX(i, j + 1)], vz[c], vz[IX(i, j + 2)], vz[IX(i, j - 1)], hz);
        real dvz_dx = D4(vz[c], vz[IX(i - 1, j)], vz[IX(i + 1, j)], vz[IX(i - 2, j)], hx);
        real dvx_dz = D4(vx[IX(i, j + 1)], vx[c], vx[IX(i, j + 2)], vx[IX(i, j - 1)], hz);
        if (pml) {
            real* m4 = a.mem[4]; real* m5 = a.mem[5]; real* m6 = a.mem[6]; real* m7 = a.mem[7];
            const real bh = bch[c], ah = ach[c], kh = kaph[c];
            const real M4 = bh * m4[c] + ah * dvx_dx;  // memory_dvx_dx2
            const real M5 = bh * m5[c] + ah * dvx_dz;  // memory_dvx_dz2
            const real M7 = bh * m7[c] + ah * dvz_dz;  // memory_dvz_dz2
            const real M6 = bh * m6[c] + ah * dvz_dx;  // memory_dvz_dx2
            m4[c] = M4; m5[c] = M5; m6[c] = M6; m7[c] = M7;
            dvx_dx = KAP(dvx_dx, kh, M4);
            dvx_dz = KAP(dvx_dz, kh, M5);
            dvz_dz = KAP(dvz_dz, kh, M7);
            dvz_dx = KAP(dvz_dx, kh, M6);
        }
        real* sxz = a.f[4];
        const real c15 = a.m[2][c], c35 = a.m[4][c], c55 = a.m[5][c];
#if SD_EXACT
        sxz[c] = (sxz[c] + (c15 * dvx_dx + c35 * dvz_dz + c55 * (dvz_dx + dvx_dz)) * dt) / (1.0 + a.m[9][c] * dt);
#else
        sxz[c] = (sxz[c] + (c15 * dvx_dx + c35 * dvz_dz + c55 * (dvz_dx + dvx_dz)) * dt) * a.m[9][c];
#endif
    }
#undef D4
}

__global__ void __launch_bounds__(BX* BY) s2_velocity(S2Args<real> a, StepInfo si) {
    const int it = *si.step;
    __shared__ double red[BX * BY / 32];
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    double nrm = 0.0;
    float sq = 0.f, n0 = 0.f, n1 = 0.f;  // FP32 build: squared norm and its components
    if (i <= nx && j <= nz) {
        const size_t c = IX(i, j);
        const real* __restrict__ sxx = a.f[2];
        const real* __restrict__ szz = a.f[3];
        const real* __restrict__ sxz = a.f[4];
        const real* __restrict__ rho = a.m[6];
        const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.k0 && j - 1 < a.box.k1);
        const real dt = a.dt;
        real vx = a.f[0][c], vz = a.f[1][c];
#if SD_EXACT
        const real hx = 24.0 * a.dx, hz = 24.0 * a.dz;
#else
        const real hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
#endif
        if (j >= 3 && j <= nz - 1 && i >= 3 && i <= nx - 1) {
            // vx, cpmlfdtd.f08:399-416: three-term stencils (reference quirk)
#if SD_EXACT
            const real rhoxx = scalar_mean_d(rho[c], rho[IX(i - 1, j)], a.density_code);
            const real rhozx = scalar_mean_d(rho[c], rho[IX(i, j - 1)], a.density_code);
            real dsxx_dx = (27.0 * sxx[c] - 27.0 * sxx[IX(i - 1, j)] + sxx[IX(i - 2, j)]) / hx;
            real dsxz_dz = (27.0 * sxz[c] - 27.0 * sxz[IX(i, j - 1)] + sxz[IX(i, j - 2)]) / hz;
#else
            const real bxx = inv_mean_f(rho[c], rho[IX(i - 1, j)], a.density_code);
            const real bzx = inv_mean_f(rho[c], rho[IX(i, j - 1)], a.density_code);
            real dsxx_dx = (27.0f * (sxx[c] - sxx[IX(i - 1, j)]) + sxx[IX(i - 2, j)]) * hx;
            real dsxz_dz = (27.0f * (sxz[c] - sxz[IX(i, j - 1)]) + sxz[IX(i, j - 2)]) * hz;
#endif
            if (pml) {
                real* m8 = a.mem[8]; real* m11 = a.mem[11];
                const real b = a.m[14][c], aa = a.m[12][c], k = a.m[10][c];
                const real M8 = b * m8[c] + aa * dsxx_dx;
                const real M11 = b * m11[c] + aa * dsxz_dz;
                m8[c] = M8; m11[c] = M11;
                dsxx_dx = KAP(dsxx_dx, k, M8);
                dsxz_dz = KAP(dsxz_dz, k, M11);
            }
#if SD_EXACT
            vx = vx + dt * (dsxx_dx / rhoxx + dsxz_dz / rhozx);
#else
            vx = vx + dt * (dsxx_dx * bxx + dsxz_dz * bzx);
#endif
        }
        if (j >= 2 && j <= nz - 2 && i >= 2 && i <= nx - 2) {
            // vz, cpmlfdtd.f08:428-446
#if SD_EXACT
            const real rhoxz = scalar_mean_d(rho[c], rho[IX(i + 1, j)], a.density_code);
            const real rhozz = scalar_mean_d(rho[c], rho[IX(i, j + 1)], a.density_code);
            real dsxz_dx = (-27.0 * sxz[c] + 27.0 * sxz[IX(i + 1, j)] - sxz[IX(i + 2, j)]) / hx;
            real dszz_dz = (-27.0 * szz[c] + 27.0 * szz[IX(i, j + 1)] - szz[IX(i, j + 2)]) / hz;
#else
            const real bxz = inv_mean_f(rho[c], rho[IX(i + 1, j)], a.density_code);
            const real bzz = inv_mean_f(rho[c], rho[IX(i, j + 1)], a.density_code);
            real dsxz_dx = (27.0f * (sxz[IX(i + 1, j)] - sxz[c]) - sxz[IX(i + 2, j)]) * hx;
            real dszz_dz = (27.0f * (szz[IX(i, j + 1)] - szz[c]) - szz[IX(i, j + 2)]) * hz;
#endif
            if (pml) {
                real* m10 = a.mem[10]; real* m9 = a.mem[9];
                const real bh = a.m[15][c], ah = a.m[13][c], kh = a.m[11][c];
                const real M10 = bh * m10[c] + ah * dsxz_dx;
                const real M9 = bh * m9[c] + ah * dszz_dz;
                m10[c] = M10; m9[c] = M9;
                dsxz_dx = KAP(dsxz_dx, kh, M10);
                dszz_dz = KAP(dszz_dz, kh, M9);
            }
#if SD_EXACT
            vz = vz + dt * (dsxz_dx / rhoxz + dszz_dz / rhozz);
#else
            vz = vz + dt * (dsxz_dx * bxz + dszz_dz * bzz);
#endif
        }
        // force source, cpmlfdtd.f08:522-523 (no dt, reference quirk)
        if (i - 1 == a.isrc && j - 1 == a.jsrc) {
            if (a.src[0]) vx = vx + (real)a.src[0][it - 1] / rho[c];
            if (a.src[1]) vz = vz + (real)a.src[1][it - 1] / rho[c];
        }
        // Dirichlet ring, cpmlfdtd.f08:534-549
        if (i == 1 || i == nx || j == 1 || j == nz) { vx = 0; vz = 0; }
        a.f[0][c] = vx;
        a.f[1][c] = vz;
#if !SD_F32
        nrm = sqrt((double)vx * (double)vx + (double)vz * (double)vz);
#else
        sq = vx * vx + vz * vz; n0 = vx; n1 = vz;
#endif
        // plane-wave face cells: their norm is taken after the injection
        if (a.pw.on && pw_cell(a.pw, i - 1, 0, j - 1)) { nrm = 0.0; sq = 0.f; n0 = 0.f; n1 = 0.f; }
    }
#if !SD_F32
    nrm = block_max<BX * BY / 32>(nrm, red);
#else
    __shared__ float redf[BX * BY / 32];
    nrm = block_norm_f32<BX * BY / 32>(sq, [&] { return sqrt((double)n0 * n0 + (double)n1 * n1); }, redf, red);
#endif
    if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(&a.norms[it - 1], nrm);
}
#undef KAP

// stress source, cpmlfdtd.f08:519-521 (applied after the velocity update)
__global__ void s2_stress_source(S2Args<real> a, StepInfo si) {
    const int it = *si.step;
    const int nx = a.nx;
    const int is = a.isrc + 1, js = a.jsrc + 1;
    const size_t c = IX(is, js), c1 = IX(is + 1, js + 1);
    const real* rho = a.m[6];
    if (a.src[2]) a.f[2][c] = a.f[2][c] + (real)a.src[2][it - 1] / rho[c];
    if (a.src[3]) a.f[4][c1] = a.f[4][c1] + (real)a.src[3][it - 1] / rho[c1];
    if (a.src[4]) a.f[3][c] = a.f[3][c] + (real)a.src[4][it - 1] / rho[c];
    (void)nx;
}

// Receiver gather (after the Dirichlet ring, like the reference's per-step
// snapshot) and advance of the device step counter; always the last
// kernel of a step.
__global__ void s2_epilogue(S2Args<real> a, StepInfo s) {
    const int it = *s.step;
    for (int r = threadIdx.x; r < s.nrec; r += blockDim.x) {
        const size_t base = (size_t)(it - 1) * 2 * s.nrec;
        a.traces[base + r] = a.f[0][s.rec[r]];
        a.traces[base + s.nrec + r] = a.f[1][s.rec[r]];
    }
    __syncthreads();
    if (threadIdx.x == 0) *s.step = it + 1;
}

}  // namespace

void SD_NAME(launch_seismic2)(const S2Args<real>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h) {
    const dim3 blk(BX, BY), grd((a.nx + BX - 1) / BX, (a.nz + BY - 1) / BY);
    s2_stress<<<grd, blk, 0, st>>>(a);
    if (h) h->fn(h->ctx, 0, "s2_stress");
    s2_velocity<<<grd, blk, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 1, "s2_velocity");
    if (a.stress_src) {
        s2_stress_source<<<1, 1, 0, st>>>(a, s);
        if (h) h->fn(h->ctx, 2, "s2_stress_source");
    }
    if (a.pw.on) pw_seismic2<real>(a, s, st);
    s2_epilogue<<<1, 256, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 3, "s2_epilogue");
}
