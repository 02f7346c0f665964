// electromag3.cu -- 3D anisotropic E/H CPML-FDTD with explicit conductivity
// (ground-penetrating radar), src/fortran/cpmlfdtd.f08:3353-4001.
//
//   e3_h : Hx, Hy (:3695-3741) and Hz (:3752-3769, from k = 2), second-order
//          forward differences of E with C-PML memories.
//   e3_e : Ex, Ey, Ez (:3787-3825) with the full conductivity tensor and the
//          inverse permittivity tensor, point source (:3901-3906), Dirichlet
//          faces (:3912-3929), max-norm (:3987-3988).
// The reference keeps Ex_old/Ey_old/Ez_old copies (:3980-3982); they always
// equal E at the start of the E update and each cell reads only its own, so
// the copies disappear.  The reference also zeroes the six H faces after the
// E update; here e3_h of the next step reads those faces as zero instead
// (same values, no extra pass), and the state copy-out zeroes them before
// reading H back.
#include "common.cuh"
#include "kernels.h"

#define IX(fi, fj, fk) \
    ((size_t)((fi) - 1) + (size_t)a.nx * ((size_t)((fj) - 1) + (size_t)a.ny * (size_t)((fk) - 1)))

namespace {
constexpr int BX = 32, BY = 8;

#if SD_EXACT
#define DIFF(p, m, h) (((p) - (m)) / (h))
#define KAP(d, k, mm) ((d) / (k) + (mm))
#else
#define DIFF(p, m, h) (((p) - (m)) * (h))  // host passes 1/h
#define KAP(d, k, mm) ((d) * (k) + (mm))   // kappa slots hold 1/kappa
#endif

__global__ void __launch_bounds__(BX* BY) e3_h(E3Args<real> a) {
    const int i = blockIdx.x * BX + threadIdx.x + 1, j = blockIdx.y * BY + threadIdx.y + 1, k = blockIdx.z + 1;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (i > nx || j > ny) return;
    const size_t c = IX(i, j, k);
    real *Hx = a.f[3], *Hy = a.f[4], *Hz = a.f[5];
    const bool face = i == 1 || i == nx || j == 1 || j == ny || k == 1 || k == nz;
    // cells the H loops never reach sit on a face: zero after every step
    if (i == nx || j == ny || k == nz) { Hx[c] = 0; Hy[c] = 0; Hz[c] = 0; return; }
    const real* __restrict__ Ex = a.f[0];
    const real* __restrict__ Ey = a.f[1];
    const real* __restrict__ Ez = a.f[2];
    const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.j0 && j - 1 < a.box.j1 &&
                       k - 1 >= a.box.k0 && k - 1 < a.box.k1);
    const real ex = Ex[c], ey = Ey[c], ez = Ez[c];
    {   // Hx, half-grid coefficients
        real dEz_dy = DIFF(Ez[IX(i, j + 1, k)], ez, a.dy);
        real dEy_dz = DIFF(Ey[IX(i, j, k + 1)], ey, a.dz);
        if (pml) {
            real *mEy_dz = a.mem[5], *mEz_dy = a.mem[4];
            const real b = a.cpml[5][c], aa = a.cpml[3][c], kk = a.cpml[1][c];
            const real M5 = b * mEy_dz[c] + aa * dEy_dz;
            const real M4 = b * mEz_dy[c] + aa * dEz_dy;
            mEy_dz[c] = M5; mEz_dy[c] = M4;
            dEz_dy = KAP(dEz_dy, kk, M4);
            dEy_dz = KAP(dEy_dz, kk, M5);
        }
        // daHx = 1 (cpmlfdtd.f08:3487): 1.0*Hx is exactly Hx
        Hx[c] = (face ? (real)0 : Hx[c]) + a.dbH * (dEy_dz - dEz_dy);
    }
    {   // Hy, full-grid coefficients
        real dEx_dz = DIFF(Ex[IX(i, j, k + 1)], ex, a.dz);
        real dEz_dx = DIFF(Ez[IX(i + 1, j, k)], ez, a.dx);
        if (pml) {
            real *mEx_dz = a.mem[2], *mEz_dx = a.mem[3];
            const real b = a.cpml[4][c], aa = a.cpml[2][c], kk = a.cpml[0][c];
            const real M2 = b * mEx_dz[c] + aa * dEx_dz;
            const real M3 = b * mEz_dx[c] + aa * dEz_dx;
            mEx_dz[c] = M2; mEz_dx[c] = M3;
            dEx_dz = KAP(dEx_dz, kk, M2);
            dEz_dx = KAP(dEz_dx, kk, M3);
        }
        Hy[c] = (face ? (real)0 : Hy[c]) + a.dbH * (dEz_dx - dEx_dz);
    }
    if (k >= 2) {  // Hz, full-grid coefficients
        real dEx_dy = DIFF(Ex[IX(i, j + 1, k)], ex, a.dy);
        real dEy_dx = DIFF(Ey[IX(i + 1, j, k)], ey, a.dx);
        if (pml) {
            real *mEx_dy = a.mem[0], *mEy_dx = a.mem[1];
            const real b = a.cpml[4][c], aa = a.cpml[2][c], kk = a.cpml[0][c];
            const real M0 = b * mEx_dy[c] + aa * dEx_dy;
            const real M1 = b * mEy_dx[c] + aa * dEy_dx;
            mEx_dy[c] = M0; mEy_dx[c] = M1;
            dEx_dy = KAP(dEx_dy, kk, M0);
            dEy_dx = KAP(dEy_dx, kk, M1);
        }
        Hz[c] = (face ? (real)0 : Hz[c]) + a.dbH * (dEx_dy - dEy_dx);
    } else {
        Hz[c] = 0;  // k = 1: face, never updated
    }
}

__global__ void __launch_bounds__(BX* BY) e3_e(E3Args<real> a, StepInfo si) {
    const int it = *si.step;
    __shared__ double red[BX * BY / 32];
    const int i = blockIdx.x * BX + threadIdx.x + 1, j = blockIdx.y * BY + threadIdx.y + 1, k = blockIdx.z + 1;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    double nrm = 0.0;
    float sq = 0.f, n0 = 0.f, n1 = 0.f, n2 = 0.f;  // FP32 build: squared norm and its components
    if (i <= nx && j <= ny) {
        const size_t c = IX(i, j, k);
        real ex = a.f[0][c], ey = a.f[1][c], ez = a.f[2][c];
        if (i >= 2 && i <= nx - 1 && j >= 2 && j <= ny - 1 && k >= 2 && k <= nz - 1) {
            const real* __restrict__ Hx = a.f[3];
            const real* __restrict__ Hy = a.f[4];
            const real* __restrict__ Hz = a.f[5];
            const real hx = Hx[c], hy = Hy[c], hz = Hz[c];
            real dHz_dy = DIFF(hz, Hz[IX(i, j - 1, k)], a.dy);
            real dHy_dz = DIFF(hy, Hy[IX(i, j, k - 1)], a.dz);
            real dHz_dx = DIFF(hz, Hz[IX(i - 1, j, k)], a.dx);
            real dHx_dz = DIFF(hx, Hx[IX(i, j, k - 1)], a.dz);
            real dHy_dx = DIFF(hy, Hy[IX(i - 1, j, k)], a.dx);
            real dHx_dy = DIFF(hx, Hx[IX(i, j - 1, k)], a.dy);
            const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && j - 1 >= a.box.j0 && j - 1 < a.box.j1 &&
                               k - 1 >= a.box.k0 && k - 1 < a.box.k1);
            if (pml) {
                const real bh = a.cpml[5][c], ah = a.cpml[3][c], kh = a.cpml[1][c];
                const real b = a.cpml[4][c], aa = a.cpml[2][c], kk = a.cpml[0][c];
                real *m6 = a.mem[6], *m7 = a.mem[7], *m8 = a.mem[8], *m9 = a.mem[9], *m10 = a.mem[10], *m11 = a.mem[11];
                const real M8 = bh * m8[c] + ah * dHz_dy;   // memory_dHz_dy
                const real M9 = b * m9[c] + aa * dHy_dz;    // memory_dHy_dz (full)
                const real M6 = bh * m6[c] + ah * dHz_dx;   // memory_dHz_dx
                const real M7 = bh * m7[c] + ah * dHx_dz;   // memory_dHx_dz
                const real M10 = bh * m10[c] + ah * dHx_dy; // memory_dHx_dy
                const real M11 = bh * m11[c] + ah * dHy_dx; // memory_dHy_dx
                m8[c] = M8; m9[c] = M9; m6[c] = M6; m7[c] = M7; m10[c] = M10; m11[c] = M11;
                dHz_dy = KAP(dHz_dy, kh, M8);
                dHy_dz = KAP(dHy_dz, kk, M9);
                dHz_dx = KAP(dHz_dx, kh, M6);
                dHx_dz = KAP(dHx_dz, kh, M7);
                dHx_dy = KAP(dHx_dy, kh, M10);
                dHy_dx = KAP(dHy_dx, kh, M11);
            }
            const real s11 = a.sig[0][c], s12 = a.sig[1][c], s13 = a.sig[2][c], s22 = a.sig[3][c],
                       s23 = a.sig[4][c], s33 = a.sig[5][c];
            const real rhs_x = dHz_dy - dHy_dz - (s11 * ex + s12 * ey + s13 * ez);
            const real rhs_y = dHx_dz - dHz_dx - (s12 * ex + s22 * ey + s23 * ez);
            const real rhs_z = dHy_dx - dHx_dy - (s13 * ex + s23 * ey + s33 * ez);
            const real exo = ex, eyo = ey, ezo = ez;
            ex = exo + (a.inv[0][c] * rhs_x + a.inv[1][c] * rhs_y + a.inv[2][c] * rhs_z) * a.dt;
            ey = eyo + (a.inv[3][c] * rhs_x + a.inv[4][c] * rhs_y + a.inv[5][c] * rhs_z) * a.dt;
            ez = ezo + (a.inv[6][c] * rhs_x + a.inv[7][c] * rhs_y + a.inv[8][c] * rhs_z) * a.dt;
        }
        if (i - 1 == a.isrc && j - 1 == a.jsrc && k - 1 == a.ksrc) {
            if (a.src[0]) ex = ex + (real)a.src[0][it - 1] * a.dt / a.eabs[0][c];
            if (a.src[1]) ey = ey + (real)a.src[1][it - 1] * a.dt / a.eabs[1][c];
            if (a.src[2]) ez = ez + (real)a.src[2][it - 1] * a.dt / a.eabs[2][c];
        }
        if (i == 1 || i == nx || j == 1 || j == ny || k == 1 || k == nz) { ex = 0; ey = 0; ez = 0; }
        a.f[0][c] = ex;
        a.f[1][c] = ey;
        a.f[2][c] = ez;
#if !SD_F32
        nrm = sqrt((double)ex * (double)ex + (double)ey * (double)ey + (double)ez * (double)ez);
#else
        sq = ex * ex + ey * ey + ez * ez; n0 = ex; n1 = ey; n2 = ez;
#endif
        // plane-wave face cells: their norm is taken after the injection
        if (a.pw.on && pw_cell(a.pw, i - 1, j - 1, k - 1)) { nrm = 0.0; sq = 0.f; n0 = n1 = n2 = 0.f; }
    }
#if !SD_F32
    nrm = block_max<BX * BY / 32>(nrm, red);
#else
    __shared__ float redf[BX * BY / 32];
    nrm = block_norm_f32<BX * BY / 32>(sq, [&] { return sqrt((double)n0 * n0 + (double)n1 * n1 + (double)n2 * n2); },
                                       redf, red);
#endif
    if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(&a.norms[it - 1], nrm);
}

// Receiver gather (Ex, Ey, Ez after the Dirichlet faces) and advance of the
// device step counter; always the last kernel of a step.
__global__ void e3_epilogue(E3Args<real> a, StepInfo s) {
    const int it = *s.step;
    for (int r = threadIdx.x; r < s.nrec; r += blockDim.x) {
        const size_t base = (size_t)(it - 1) * 3 * s.nrec;
        a.traces[base + r] = a.f[0][s.rec[r]];
        a.traces[base + s.nrec + r] = a.f[1][s.rec[r]];
        a.traces[base + 2 * s.nrec + r] = a.f[2][s.rec[r]];
    }
    __syncthreads();
    if (threadIdx.x == 0) *s.step = it + 1;
}
#undef DIFF
#undef KAP
}  // namespace

void SD_NAME(launch_electromag3)(const E3Args<real>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h) {
    const dim3 blk(BX, BY), grd((a.nx + BX - 1) / BX, (a.ny + BY - 1) / BY, a.nz);
    e3_h<<<grd, blk, 0, st>>>(a);
    if (h) h->fn(h->ctx, 0, "e3_h");
    e3_e<<<grd, blk, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 1, "e3_e");
    if (a.pw.on) pw_electromag3<real>(a, s, st);
    e3_epilogue<<<1, 256, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 2, "e3_epilogue");
}
