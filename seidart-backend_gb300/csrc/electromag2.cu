// electromag2.cu -- 2D anisotropic E/H (TE: Ex, Ez, Hy) CPML-FDTD with
// explicit conductivity, src/fortran/cpmlfdtd.f08:2566-2748.
//
//   e2_h : Hy update (:2576-2593), second-order differences with CPML.
//   e2_e : Ex, Ez update (:2605-2620), point source (:2678-2681), Dirichlet
//          ring on Ex/Ez (:2690-2707), max-norm (:2726-2740).
// The reference keeps Ex_old/Ez_old copies (:2711-2716); they always equal
// Ex/Ez at the start of the E update, so each thread reads its cell once and
// the two extra full-grid passes per step disappear.
// The reference also zeroes the Hy ring after the E update.  Here e2_h of the
// next step reads the ring as zero instead (same values, one launch fewer);
// the state copy-out zeroes the ring before reading Hy back.
#include "common.cuh"
#include "kernels.h"

#define IX(fi, fk) ((size_t)((fi) - 1) + (size_t)a.nx * (size_t)((fk) - 1))

namespace {
constexpr int BX = 32, BY = 8;

__global__ void __launch_bounds__(BX* BY) e2_h(E2Args<real> a) {
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    if (i > nx || j > nz) return;
    const size_t c = IX(i, j);
    real* Hy = a.f[2];
    const bool ring = (i == 1 || i == nx || j == 1 || j == nz);
    if (i == nx || j == nz) { Hy[c] = 0; return; }
    const real* __restrict__ Ex = a.f[0];
    const real* __restrict__ Ez = a.f[1];
#if SD_EXACT
    real dEx_dz = (Ex[IX(i, j + 1)] - Ex[c]) / a.dz;
    real dEz_dx = (Ez[IX(i + 1, j)] - Ez[c]) / a.dx;
#else
    real dEx_dz = (Ex[IX(i, j + 1)] - Ex[c]) * a.dz;  // host passes 1/dz, 1/dx
    real dEz_dx = (Ez[IX(i + 1, j)] - Ez[c]) * a.dx;
#endif
    const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.k0 && j - 1 < a.box.k1);
    if (pml) {
        real* m0 = a.mem[0];  // memory_dEx_dz
        real* m1 = a.mem[1];  // memory_dEz_dx
        const real M0 = a.cpml[4][c] * m0[c] + a.cpml[2][c] * dEx_dz;
        const real M1 = a.cpml[5][c] * m1[c] + a.cpml[3][c] * dEz_dx;
        m0[c] = M0; m1[c] = M1;
#if SD_EXACT
        dEz_dx = dEz_dx / a.cpml[1][c] + M1;
        dEx_dz = dEx_dz / a.cpml[0][c] + M0;
#else
        dEz_dx = dEz_dx * a.cpml[1][c] + M1;
        dEx_dz = dEx_dz * a.cpml[0][c] + M0;
#endif
    }
    const real hy = ring ? (real)0 : Hy[c];
    // daHy = 1 (cpmlfdtd.f08:2521): 1.0*Hy is exactly Hy
    Hy[c] = hy + a.dbHy * (dEz_dx - dEx_dz);
}

__global__ void __launch_bounds__(BX* BY) e2_e(E2Args<real> a, StepInfo si) {
    const int it = *si.step;
    __shared__ double red[BX * BY / 32];
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    double nrm = 0.0;
    float sq = 0.f, n0 = 0.f, n1 = 0.f;  // FP32 build: squared norm and its components
    if (i <= nx && j <= nz) {
        const size_t c = IX(i, j);
        real ex = a.f[0][c], ez = a.f[1][c];
        if (i >= 2 && j >= 2) {
            const real* __restrict__ Hy = a.f[2];
#if SD_EXACT
            real dHy_dz = (Hy[c] - Hy[IX(i, j - 1)]) / a.dz;
            real dHy_dx = (Hy[c] - Hy[IX(i - 1, j)]) / a.dx;
#else
            real dHy_dz = (Hy[c] - Hy[IX(i, j - 1)]) * a.dz;
            real dHy_dx = (Hy[c] - Hy[IX(i - 1, j)]) * a.dx;
#endif
            const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.k0 && j - 1 < a.box.k1);
            if (pml) {
                real* m2 = a.mem[2];  // memory_dHy_dx
                real* m3 = a.mem[3];  // memory_dHy_dz
                const real M2 = a.cpml[5][c] * m2[c] + a.cpml[3][c] * dHy_dx;
                const real M3 = a.cpml[4][c] * m3[c] + a.cpml[2][c] * dHy_dz;
                m2[c] = M2; m3[c] = M3;
#if SD_EXACT
                dHy_dz = dHy_dz / a.cpml[0][c] + M3;
                dHy_dx = dHy_dx / a.cpml[1][c] + M2;
#else
                dHy_dz = dHy_dz * a.cpml[0][c] + M3;
                dHy_dx = dHy_dx * a.cpml[1][c] + M2;
#endif
            }
            const real aEx = a.c[0][c], bEx = a.c[1][c], dEx = a.c[2][c], eEx = a.c[3][c];
            const real aEz = a.c[4][c], bEz = a.c[5][c], dEz = a.c[6][c], eEz = a.c[7][c];
            const real exo = ex, ezo = ez;
            ez = ezo + (-(aEz * dHy_dz) + bEz * dHy_dx - dEz * exo - eEz * ezo) * a.dt;
            ex = exo + (-(aEx * dHy_dz) + bEx * dHy_dx - dEx * exo - eEx * ezo) * a.dt;
        }
        if (i - 1 == a.isrc && j - 1 == a.jsrc) {
            if (a.src[0]) ex = ex + (real)a.src[0][it - 1] * a.dt / a.c[8][c];
            if (a.src[1]) ez = ez + (real)a.src[1][it - 1] * a.dt / a.c[9][c];
        }
        if (i == 1 || i == nx || j == 1 || j == nz) { ex = 0; ez = 0; }
        a.f[0][c] = ex;
        a.f[1][c] = ez;
#if !SD_F32
        nrm = sqrt((double)ex * (double)ex + (double)ez * (double)ez);
#else
        sq = ex * ex + ez * ez; n0 = ex; n1 = ez;
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

// Receiver gather (after the Dirichlet ring, like the reference's per-step
// snapshot) and advance of the device step counter; always the last
// kernel of a step.
__global__ void e2_epilogue(E2Args<real> a, StepInfo s) {
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

void SD_NAME(launch_electromag2)(const E2Args<real>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h) {
    const dim3 blk(BX, BY), grd((a.nx + BX - 1) / BX, (a.nz + BY - 1) / BY);
    e2_h<<<grd, blk, 0, st>>>(a);
    if (h) h->fn(h->ctx, 0, "e2_h");
    e2_e<<<grd, blk, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 1, "e2_e");
    if (a.pw.on) pw_electromag2<real>(a, s, st);
    e2_epilogue<<<1, 256, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 2, "e2_epilogue");
}
