// adjoint.cu -- misfit gradient of the 2D elastic solver by a hand-written
// discrete adjoint (full-waveform inversion of seismic2,
// src/fortran/cpmlfdtd.f08:311-576, FP32 fields).
//
// One forward step x_{n-1} -> x_n (state x = vx, vz, sigma_xx, sigma_zz,
// sigma_xz and the 12 CPML memories) is the composition
//     stress half-step S, velocity half-step V, force source, Dirichlet ring D
// exactly as seismic2.cu computes it in FP32.  For the loss
//     L = 1/2 sum_n sum_receivers |v_n(r) - d_n(r)|^2
// the adjoint sweep runs n = N .. 1:
//     lambda += dL/dv_n at the receivers;  lambda <- S^T V^T D^T lambda
// where the transposes are written out by hand for the implemented operator:
// CPML recursions (m' = b m + a d, d' = d/kappa + m'), attenuation
// 1/(1 + gamma dt), the three-term velocity stencils, loop bounds and the
// Dirichlet ring.  Gradients accumulate in FP64 per cell:
//     dL/dc11, dL/dc13, dL/dc33, dL/dc55 from S, and the four face
//     buoyancies of V (chained to rho on the host, plus the source term).
// Memory: forward states are kept every K ~ sqrt(nt) steps; the sweep
// recomputes one K-step segment at a time from its checkpoint and walks it
// backwards (storage ~2 sqrt(nt) states, cost ~1 extra forward).
// Launches: per shot, one CUDA graph recomputes a K-step segment (saving
// every state) and one walks it backwards; the step numbers come from a
// device-side segment base, so the same two graphs replay for every segment
// and a segment costs four host operations.  An adjoint step is two grid
// passes: adj_velocity (receiver residuals, the gather of S^T left by the
// step after, D^T, V^T) and adj_stress (gather of V^T, S^T).
// The same driver runs the electromag2 adjoint (adjoint_em.cu) with a
// 7-array state; the family decides the kernels and the gradient chain.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/seidart_gpu.h"
#include "common.cuh"
#include "kernels.h"
#include "trace.h"

extern "C" int seidart_solver_internal_s2f(SeidartSolver* s, S2Args<float>* out, const int** rec);
extern "C" int seidart_solver_internal_e2f(SeidartSolver* s, E2Args<float>* out, const int** rec);
extern "C" int seidart_solver_internal_reset(SeidartSolver* s);
extern "C" int seidart_solver_internal_share_model(SeidartSolver* dst, const SeidartSolver* src);
extern "C" int seidart_solver_internal_advance(SeidartSolver* s, int nsteps);
extern "C" int seidart_solver_internal_set_step(SeidartSolver* s, int steps_done);
extern "C" int seidart_solver_internal_set_source(SeidartSolver* s, int isrc, int jsrc, const double* dev_srcx,
                                                  const double* dev_srcz);
extern "C" cudaStream_t seidart_solver_internal_stream(SeidartSolver* s);
extern "C" StepInfo seidart_solver_internal_stepinfo(SeidartSolver* s);

namespace {

constexpr int BX = 32, BY = 8;
constexpr int NS = 17;  // seismic2 state arrays: vx vz sxx szz sxz M0..M11
constexpr int NS_EM = 7;  // electromag2 state arrays: Ex Ez Hy M0..M3

struct AdjArgs {
    int nx, nz, density_code;
    float dt, hx, hz;  // hx = 1/(24 dx)
    BoxH box;
    const float* m[16];  // FP32 model: c11 c13 c15 c33 c35 c55 rho gx gz gxz 1/k 1/kh a ah b bh
    const float* xp;     // x_{n-1}, NS arrays of N
    const float* xc;     // x_n
    float* lam;          // adjoint state, NS arrays
    float* scr;          // 12 scratch arrays: lf1..lf4, ld1..ld4, le1..le4
    float* grad;         // FP32 accumulators of the current segment: c11 c13 c33 c55 Bxx Bzx Bxz Bzz
                         // (and c15 c35 when `full`)
    int full;            // 1: also dL/dc15 and dL/dc35 (slots 8, 9)
    size_t N;
    int isrc, jsrc;
    const double* srcz;  // force series of the shot (device), NULL = none
    const int* base;     // device: steps before the segment; this step is n = *base + j
    int j;
    double* gsrc;        // accumulated lambda_vz(src) * f_n
    // receiver residuals dL/dv_n, added where a cell holds receivers:
    // rfirst[c] = first receiver at cell c (-1: none), rnext[r] = next one
    const int* rfirst;
    const int* rnext;
    const float* dres;   // [nt][2][nrec], NULL = no residual (test hook)
    int nrec;
};

__device__ __forceinline__ bool inN(int i, int k, int nx, int nz) { return k >= 2 && k <= nz - 2 && i >= 1 && i <= nx - 3; }
__device__ __forceinline__ bool inS(int i, int k, int nx, int nz) { return k >= 1 && k <= nz - 3 && i >= 2 && i <= nx - 2; }
__device__ __forceinline__ bool inX(int i, int k, int nx, int nz) { return k >= 2 && k <= nz - 2 && i >= 2 && i <= nx - 2; }
__device__ __forceinline__ bool inZ(int i, int k, int nx, int nz) { return k >= 1 && k <= nz - 3 && i >= 1 && i <= nx - 3; }

// value of array a at (i, k), zero outside the grid
__device__ __forceinline__ float at(const float* a, int i, int k, int nx, int nz) {
    return (i >= 0 && i < nx && k >= 0 && k < nz) ? a[(size_t)i + (size_t)nx * k] : 0.0f;
}

// ---------------------------------------------------------------- V^T (and D^T)
// transposes of forward (F) and backward (B) 4th-order differences, the
// gather of S^T of the step after this one into vx, vz
__device__ __forceinline__ void gather_sT(const AdjArgs& A, int i, int k, float& gvx, float& gvz) {
    const int nx = A.nx, nz = A.nz;
    const size_t N = A.N;
    const float hx = A.hx, hz = A.hz;
    const float* s = A.scr + 4 * N;
    const float *ld1 = s, *ld2 = s + N, *ld3 = s + 2 * N, *ld4 = s + 3 * N;
    const float *le1 = s + 4 * N, *le2 = s + 5 * N, *le3 = s + 6 * N, *le4 = s + 7 * N;
    auto FxT = [&](const float* d) {
        return hx * (27.0f * at(d, i - 1, k, nx, nz) - 27.0f * at(d, i, k, nx, nz) - at(d, i - 2, k, nx, nz) +
                     at(d, i + 1, k, nx, nz));
    };
    auto BxT = [&](const float* d) {
        return hx * (27.0f * at(d, i, k, nx, nz) - 27.0f * at(d, i + 1, k, nx, nz) - at(d, i - 1, k, nx, nz) +
                     at(d, i + 2, k, nx, nz));
    };
    auto FzT = [&](const float* d) {
        return hz * (27.0f * at(d, i, k - 1, nx, nz) - 27.0f * at(d, i, k, nx, nz) - at(d, i, k - 2, nx, nz) +
                     at(d, i, k + 1, nx, nz));
    };
    auto BzT = [&](const float* d) {
        return hz * (27.0f * at(d, i, k, nx, nz) - 27.0f * at(d, i, k + 1, nx, nz) - at(d, i, k - 1, nx, nz) +
                     at(d, i, k + 2, nx, nz));
    };
    gvx = FxT(ld1) + BzT(ld4) + BxT(le1) + FzT(le4);
    gvz = BzT(ld2) + FxT(ld3) + FzT(le2) + BxT(le3);
}

// Starts the adjoint of step n: completes lambda_v(n) (gather of S^T from
// step n+1, receiver residuals of step n), then D^T and V^T.  Every load
// precedes the first store: a store to one array would otherwise hold every
// later load behind it (the compiler cannot rule out aliasing between the
// slices of lam, grad and scr), one DRAM round trip each.
__global__ void __launch_bounds__(BX* BY) adj_velocity(AdjArgs A) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const int nx = A.nx, nz = A.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = A.N;
    float* lam = A.lam;
    float gvx, gvz;
    gather_sT(A, i, k, gvx, gvz);
    float lvx = lam[c] + gvx, lvz = lam[N + c] + gvz;
    if (A.dres) {
        const float* res = A.dres + (size_t)(*A.base + A.j - 1) * 2 * A.nrec;
        for (int r = A.rfirst[c]; r >= 0; r = A.rnext[r]) {
            lvx += res[r];
            lvz += res[A.nrec + r];
        }
    }
    if (i == 0 || i == nx - 1 || k == 0 || k == nz - 1) {  // D^T
        lvx = 0.f;
        lvz = 0.f;
    }
    const float* xc = A.xc;
    const float *sxx = xc + 2 * N, *szz = xc + 3 * N, *sxz = xc + 4 * N;
    const float* rho = A.m[6];
    const bool pml = !(i >= A.box.i0 && i < A.box.i1 && k >= A.box.k0 && k < A.box.k1);
    const float dt = A.dt, hx = A.hx, hz = A.hz;
    const bool ix = inX(i, k, nx, nz), iz = inZ(i, k, nx, nz);
    float lf1 = 0.f, lf2 = 0.f, lf3 = 0.f, lf4 = 0.f;
    float l8 = 0.f, l11 = 0.f, l10 = 0.f, l9 = 0.f, g4 = 0.f, g5 = 0.f, g6 = 0.f, g7 = 0.f;
    if (ix) {
        const float bxx = inv_mean_f(rho[c], rho[c - 1], A.density_code);
        const float bzx = inv_mean_f(rho[c], rho[c - nx], A.density_code);
        float F1 = (27.0f * (sxx[c] - sxx[c - 1]) + sxx[c - 2]) * hx;
        float F2 = (27.0f * (sxz[c] - sxz[c - nx]) + sxz[c - 2 * nx]) * hz;
        const float p1 = dt * bxx * lvx, p2 = dt * bzx * lvx;
        if (pml) {
            const float ik = A.m[10][c], a = A.m[12][c], b = A.m[14][c];
            F1 = F1 * ik + xc[(5 + 8) * N + c];
            F2 = F2 * ik + xc[(5 + 11) * N + c];
            const float o8 = lam[(5 + 8) * N + c], o11 = lam[(5 + 11) * N + c];
            lf1 = (ik + a) * p1 + a * o8;
            l8 = b * (p1 + o8);
            lf2 = (ik + a) * p2 + a * o11;
            l11 = b * (p2 + o11);
        } else {
            lf1 = p1;
            lf2 = p2;
        }
        g4 = A.grad[4 * N + c] + lvx * dt * F1;
        g5 = A.grad[5 * N + c] + lvx * dt * F2;
    }
    if (iz) {
        const float bxz = inv_mean_f(rho[c], rho[c + 1], A.density_code);
        const float bzz = inv_mean_f(rho[c], rho[c + nx], A.density_code);
        float F3 = (27.0f * (sxz[c + 1] - sxz[c]) - sxz[c + 2]) * hx;
        float F4 = (27.0f * (szz[c + nx] - szz[c]) - szz[c + 2 * nx]) * hz;
        const float p3 = dt * bxz * lvz, p4 = dt * bzz * lvz;
        if (pml) {
            const float ikh = A.m[11][c], ah = A.m[13][c], bh = A.m[15][c];
            F3 = F3 * ikh + xc[(5 + 10) * N + c];
            F4 = F4 * ikh + xc[(5 + 9) * N + c];
            const float o10 = lam[(5 + 10) * N + c], o9 = lam[(5 + 9) * N + c];
            lf3 = (ikh + ah) * p3 + ah * o10;
            l10 = bh * (p3 + o10);
            lf4 = (ikh + ah) * p4 + ah * o9;
            l9 = bh * (p4 + o9);
        } else {
            lf3 = p3;
            lf4 = p4;
        }
        g6 = A.grad[6 * N + c] + lvz * dt * F3;
        g7 = A.grad[7 * N + c] + lvz * dt * F4;
    }
    const bool src = i == A.isrc && k == A.jsrc && A.srcz;
    const double fsrc = src ? (double)(float)A.srcz[*A.base + A.j - 1] : 0.0;
    // ---- stores
    lam[c] = lvx;
    lam[N + c] = lvz;
    if (src) *A.gsrc += (double)lvz * fsrc;
    if (ix) {
        if (pml) {
            lam[(5 + 8) * N + c] = l8;
            lam[(5 + 11) * N + c] = l11;
        }
        A.grad[4 * N + c] = g4;
        A.grad[5 * N + c] = g5;
    }
    if (iz) {
        if (pml) {
            lam[(5 + 10) * N + c] = l10;
            lam[(5 + 9) * N + c] = l9;
        }
        A.grad[6 * N + c] = g6;
        A.grad[7 * N + c] = g7;
    }
    A.scr[c] = lf1;
    A.scr[N + c] = lf2;
    A.scr[2 * N + c] = lf3;
    A.scr[3 * N + c] = lf4;
}

// ------------------------------------------------- gather of V^T, then S^T
// All loads first, then all stores (as in adj_velocity).
__global__ void __launch_bounds__(BX* BY) adj_stress(AdjArgs A) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const int nx = A.nx, nz = A.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = A.N;
    const float hx = A.hx, hz = A.hz, dt = A.dt;
    const float *lf1 = A.scr, *lf2 = A.scr + N, *lf3 = A.scr + 2 * N, *lf4 = A.scr + 3 * N;
    // transposes of the three-term velocity stencils
    const float lsxx = A.lam[2 * N + c] +
                       hx * (27.0f * at(lf1, i, k, nx, nz) - 27.0f * at(lf1, i + 1, k, nx, nz) + at(lf1, i + 2, k, nx, nz));
    const float lsxz = A.lam[4 * N + c] +
                       hz * (27.0f * at(lf2, i, k, nx, nz) - 27.0f * at(lf2, i, k + 1, nx, nz) + at(lf2, i, k + 2, nx, nz)) +
                       hx * (-27.0f * at(lf3, i, k, nx, nz) + 27.0f * at(lf3, i - 1, k, nx, nz) - at(lf3, i - 2, k, nx, nz));
    const float lszz = A.lam[3 * N + c] +
                       hz * (-27.0f * at(lf4, i, k, nx, nz) + 27.0f * at(lf4, i, k - 1, nx, nz) - at(lf4, i, k - 2, nx, nz));
    const bool pml = !(i >= A.box.i0 && i < A.box.i1 && k >= A.box.k0 && k < A.box.k1);
    const float* const* m = A.m;
    const float* vx = A.xp;
    const float* vz = A.xp + N;
    const float* xc = A.xc;
    float* lam = A.lam;
    const bool in_n = inN(i, k, nx, nz), in_s = inS(i, k, nx, nz);
    float ld1 = 0.f, ld2 = 0.f, ld3 = 0.f, ld4 = 0.f, le1 = 0.f, le2 = 0.f, le3 = 0.f, le4 = 0.f;
    float nsxx = lsxx, nszz = lszz, nsxz = lsxz;
    float l0 = 0.f, l1 = 0.f, l2 = 0.f, l3 = 0.f, l4 = 0.f, l5 = 0.f, l6 = 0.f, l7 = 0.f;  // new memory adjoints
    float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;  // new gradient sums
    // dL/dc15, dL/dc35 collect a term from each loop, normal loop first
    const bool full = A.full && (in_n || in_s);
    float g8 = full ? A.grad[8 * N + c] : 0.f, g9 = full ? A.grad[9 * N + c] : 0.f;
    if (in_n) {
        const float gx = m[7][c], gz = m[8][c];
        const float px = dt * gx * lsxx, pz = dt * gz * lszz;
        nsxx = gx * lsxx;
        nszz = gz * lszz;
        // forward rescaled derivatives of this step (for the gradients)
        float D1 = (27.0f * (vx[c + 1] - vx[c]) - (vx[c + 2] - vx[c - 1])) * hx;
        float D2 = (27.0f * (vz[c] - vz[c - nx]) - (vz[c + nx] - vz[c - 2 * nx])) * hz;
        const float c11 = m[0][c], c13 = m[1][c], c15 = m[2][c], c33 = m[3][c], c35 = m[4][c];
        float lD1 = c11 * px + c13 * pz, lD2 = c13 * px + c33 * pz, lD3 = c15 * px + c35 * pz;
        if (pml) {
            const float ik = m[10][c], ikh = m[11][c], a = m[12][c], ah = m[13][c], b = m[14][c], bh = m[15][c];
            D1 = D1 * ikh + xc[(5 + 0) * N + c];
            D2 = D2 * ik + xc[(5 + 3) * N + c];
            const float o0 = lam[(5 + 0) * N + c];  // dvx_dx1 (half)
            const float o1 = lam[(5 + 1) * N + c];  // dvx_dz1 (half)
            const float o3 = lam[(5 + 3) * N + c];  // dvz_dz1 (full)
            const float o2 = lam[(5 + 2) * N + c];  // dvz_dx1 (full)
            ld1 = (ikh + ah) * lD1 + ah * o0;
            l0 = bh * (lD1 + o0);
            ld4 = (ikh + ah) * lD3 + ah * o1;
            l1 = bh * (lD3 + o1);
            ld2 = (ik + a) * lD2 + a * o3;
            l3 = b * (lD2 + o3);
            ld3 = (ik + a) * lD3 + a * o2;
            l2 = b * (lD3 + o2);
        } else {
            ld1 = lD1;
            ld2 = lD2;
            ld3 = lD3;
            ld4 = lD3;
        }
        g0 = A.grad[c] + px * D1;
        g1 = A.grad[N + c] + (px * D2 + pz * D1);
        g2 = A.grad[2 * N + c] + pz * D2;
        if (A.full) {
            // c15 and c35 multiply dvz_dx + dvx_dz of the normal-stress loop
            // (cpmlfdtd.f08:342-351): forward x (full coefficients) and
            // backward z (half coefficients), C-PML rescaled as the step did
            float D3 = (27.0f * (vz[c + 1] - vz[c]) - (vz[c + 2] - vz[c - 1])) * hx;
            float D4 = (27.0f * (vx[c] - vx[c - nx]) - (vx[c + nx] - vx[c - 2 * nx])) * hz;
            if (pml) {
                D3 = D3 * m[10][c] + xc[(5 + 2) * N + c];
                D4 = D4 * m[11][c] + xc[(5 + 1) * N + c];
            }
            g8 = g8 + px * (D3 + D4);
            g9 = g9 + pz * (D3 + D4);
        }
    }
    if (in_s) {
        const float gxz = m[9][c];
        const float pxz = dt * gxz * lsxz;
        nsxz = gxz * lsxz;
        float E3 = (27.0f * (vz[c] - vz[c - 1]) - (vz[c + 1] - vz[c - 2])) * hx;
        float E4 = (27.0f * (vx[c + nx] - vx[c]) - (vx[c + 2 * nx] - vx[c - nx])) * hz;
        const float lE1 = m[2][c] * pxz, lE2 = m[4][c] * pxz, lE34 = m[5][c] * pxz;
        if (pml) {
            const float ikh = m[11][c], ah = m[13][c], bh = m[15][c];
            E3 = E3 * ikh + xc[(5 + 6) * N + c];
            E4 = E4 * ikh + xc[(5 + 5) * N + c];
            const float o4 = lam[(5 + 4) * N + c];  // dvx_dx2
            const float o5 = lam[(5 + 5) * N + c];  // dvx_dz2
            const float o6 = lam[(5 + 6) * N + c];  // dvz_dx2
            const float o7 = lam[(5 + 7) * N + c];  // dvz_dz2
            le1 = (ikh + ah) * lE1 + ah * o4;
            l4 = bh * (lE1 + o4);
            le4 = (ikh + ah) * lE34 + ah * o5;
            l5 = bh * (lE34 + o5);
            le3 = (ikh + ah) * lE34 + ah * o6;
            l6 = bh * (lE34 + o6);
            le2 = (ikh + ah) * lE2 + ah * o7;
            l7 = bh * (lE2 + o7);
        } else {
            le1 = lE1;
            le2 = lE2;
            le3 = lE34;
            le4 = lE34;
        }
        g3 = A.grad[3 * N + c] + pxz * (E3 + E4);
        if (A.full) {
            // sigma_xz's c15 dvx_dx (backward x) and c35 dvz_dz (forward z),
            // half coefficients (cpmlfdtd.f08:380-383)
            float E1 = (27.0f * (vx[c] - vx[c - 1]) - (vx[c + 1] - vx[c - 2])) * hx;
            float E2 = (27.0f * (vz[c + nx] - vz[c]) - (vz[c + 2 * nx] - vz[c - nx])) * hz;
            if (pml) {
                const float ikh = m[11][c];
                E1 = E1 * ikh + xc[(5 + 4) * N + c];
                E2 = E2 * ikh + xc[(5 + 7) * N + c];
            }
            g8 = g8 + pxz * E1;
            g9 = g9 + pxz * E2;
        }
    }
    // ---- stores
    lam[2 * N + c] = nsxx;
    lam[3 * N + c] = nszz;
    lam[4 * N + c] = nsxz;
    if (in_n) {
        if (pml) {
            lam[(5 + 0) * N + c] = l0;
            lam[(5 + 1) * N + c] = l1;
            lam[(5 + 3) * N + c] = l3;
            lam[(5 + 2) * N + c] = l2;
        }
        A.grad[c] = g0;
        A.grad[N + c] = g1;
        A.grad[2 * N + c] = g2;
    }
    if (in_s) {
        if (pml) {
            lam[(5 + 4) * N + c] = l4;
            lam[(5 + 5) * N + c] = l5;
            lam[(5 + 6) * N + c] = l6;
            lam[(5 + 7) * N + c] = l7;
        }
        A.grad[3 * N + c] = g3;
    }
    if (full) {
        A.grad[8 * N + c] = g8;
        A.grad[9 * N + c] = g9;
    }
    float* s = A.scr + 4 * N;
    s[c] = ld1; s[N + c] = ld2; s[2 * N + c] = ld3; s[3 * N + c] = ld4;
    s[4 * N + c] = le1; s[5 * N + c] = le2; s[6 * N + c] = le3; s[7 * N + c] = le4;
}

// pending gather of S^T into vx, vz (host test hook only; the sweep leaves
// it to the next step's adj_velocity)
__global__ void __launch_bounds__(BX* BY) adj_flush_v(AdjArgs A) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    if (i >= A.nx || k >= A.nz) return;
    const size_t c = (size_t)i + (size_t)A.nx * k;
    float gvx, gvz;
    gather_sT(A, i, k, gvx, gvz);
    A.lam[c] += gvx;
    A.lam[A.N + c] += gvz;
}

// residual r = traces - observed over all steps; loss += 1/2 sum r^2 (FP64)
__global__ void residual_loss(const float* tr, const float* obs, float* res, size_t n, double* loss) {
    __shared__ double red[8];
    double acc = 0.0;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const float r = tr[q] - obs[q];
        res[q] = r;
        acc += (double)r * (double)r;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        atomicAdd(loss, 0.5 * t);
    }
}

// gather/scatter of the 17 state arrays between a solver and a contiguous block
struct StatePtrs {
    float* p[NS];
};
// start of a recomputed segment: solver step counter and segment base
__global__ void seg_begin(int* step, int* base, int t0) {
    *step = t0 + 1;
    *base = t0;
}

__global__ void copy_state(StatePtrs s, float* blk, size_t N, int to_block, int ns) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < N; q += (size_t)gridDim.x * blockDim.x) {
        for (int a = 0; a < ns; ++a) {
            if (to_block) blk[a * N + q] = s.p[a][q];
            else s.p[a][q] = blk[a * N + q];
        }
    }
}

// ------------------------------------------- out-of-place recompute step
// One forward step of the FP32 solver (the arithmetic of seismic2.cu's FP32
// build, stress then velocity) reading state x_{j-1} from `in` and writing
// x_j to `out`, so a recomputed segment needs no state copies.  Only cells a
// step updates are written: every other cell of a segment buffer holds zero
// from its allocation, as it does in the in-place solver (fields outside the
// loops, memories outside the CPML shell).  Fields outside the loops are
// copied through, so a restored checkpoint carries over unchanged.
struct OopArgs {
    S2Args<float> a;     // model, sizes, source position
    const float* in;     // x_{j-1}: [NS][N]
    float* out;          // x_j
    size_t N;
    const double* srcz;  // force series of the shot (device), NULL = none
    const int* base;     // device: steps before the segment; this step is *base + j
    int j;
};

#define D4F(p1, p0, p2, m1, h) ((27.0f * ((p1) - (p0)) - ((p2) - (m1))) * (h))

// Both recompute kernels issue every load before the first store (the
// slices of `in` and `out` could alias as far as the compiler knows).
__global__ void __launch_bounds__(BX* BY) oop_stress(OopArgs O) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const S2Args<float>& a = O.a;
    const int nx = a.nx, nz = a.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = O.N;
    const float *vx = O.in, *vz = O.in + N;
    const float* mi = O.in + 5 * N;
    float* mo = O.out + 5 * N;
    const bool normal = inN(i, k, nx, nz), shear = inS(i, k, nx, nz);
    const bool pml = !(i >= a.box.i0 && i < a.box.i1 && k >= a.box.k0 && k < a.box.k1);
    const float dt = a.dt;
    const float hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
    float sxx = O.in[2 * N + c], szz = O.in[3 * N + c], sxz = O.in[4 * N + c];
    float M0 = 0.f, M1 = 0.f, M2 = 0.f, M3 = 0.f, M4 = 0.f, M5 = 0.f, M6 = 0.f, M7 = 0.f;
    if (normal) {
        float dvx_dx = D4F(vx[c + 1], vx[c], vx[c + 2], vx[c - 1], hx);
        float dvz_dz = D4F(vz[c], vz[c - nx], vz[c + nx], vz[c - 2 * nx], hz);
        float dvz_dx = D4F(vz[c + 1], vz[c], vz[c + 2], vz[c - 1], hx);
        float dvx_dz = D4F(vx[c], vx[c - nx], vx[c + nx], vx[c - 2 * nx], hz);
        if (pml) {
            const float bh = a.m[15][c], ah = a.m[13][c], b = a.m[14][c], aa = a.m[12][c];
            M0 = bh * mi[c] + ah * dvx_dx;
            M1 = bh * mi[N + c] + ah * dvx_dz;
            M3 = b * mi[3 * N + c] + aa * dvz_dz;
            M2 = b * mi[2 * N + c] + aa * dvz_dx;
            dvx_dx = dvx_dx * a.m[11][c] + M0;
            dvx_dz = dvx_dz * a.m[11][c] + M1;
            dvz_dz = dvz_dz * a.m[10][c] + M3;
            dvz_dx = dvz_dx * a.m[10][c] + M2;
        }
        const float c11 = a.m[0][c], c13 = a.m[1][c], c15 = a.m[2][c], c33 = a.m[3][c], c35 = a.m[4][c];
        sxx = (sxx + (c11 * dvx_dx + c13 * dvz_dz + c15 * (dvz_dx + dvx_dz)) * dt) * a.m[7][c];
        szz = (szz + (c13 * dvx_dx + c33 * dvz_dz + c35 * (dvz_dx + dvx_dz)) * dt) * a.m[8][c];
    }
    if (shear) {
        float dvx_dx = D4F(vx[c], vx[c - 1], vx[c + 1], vx[c - 2], hx);
        float dvz_dz = D4F(vz[c + nx], vz[c], vz[c + 2 * nx], vz[c - nx], hz);
        float dvz_dx = D4F(vz[c], vz[c - 1], vz[c + 1], vz[c - 2], hx);
        float dvx_dz = D4F(vx[c + nx], vx[c], vx[c + 2 * nx], vx[c - nx], hz);
        if (pml) {
            const float bh = a.m[15][c], ah = a.m[13][c], kh = a.m[11][c];
            M4 = bh * mi[4 * N + c] + ah * dvx_dx;
            M5 = bh * mi[5 * N + c] + ah * dvx_dz;
            M7 = bh * mi[7 * N + c] + ah * dvz_dz;
            M6 = bh * mi[6 * N + c] + ah * dvz_dx;
            dvx_dx = dvx_dx * kh + M4;
            dvx_dz = dvx_dz * kh + M5;
            dvz_dz = dvz_dz * kh + M7;
            dvz_dx = dvz_dx * kh + M6;
        }
        const float c15 = a.m[2][c], c35 = a.m[4][c], c55 = a.m[5][c];
        sxz = (sxz + (c15 * dvx_dx + c35 * dvz_dz + c55 * (dvz_dx + dvx_dz)) * dt) * a.m[9][c];
    }
    // ---- stores (fields outside the loops are copied through)
    O.out[2 * N + c] = sxx;
    O.out[3 * N + c] = szz;
    O.out[4 * N + c] = sxz;
    if (pml && normal) { mo[c] = M0; mo[N + c] = M1; mo[2 * N + c] = M2; mo[3 * N + c] = M3; }
    if (pml && shear) { mo[4 * N + c] = M4; mo[5 * N + c] = M5; mo[6 * N + c] = M6; mo[7 * N + c] = M7; }
}

__global__ void __launch_bounds__(BX* BY) oop_velocity(OopArgs O) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const S2Args<float>& a = O.a;
    const int nx = a.nx, nz = a.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = O.N;
    const float *sxx = O.out + 2 * N, *szz = O.out + 3 * N, *sxz = O.out + 4 * N;  // sigma of step j
    const float* mi = O.in + 5 * N;
    float* mo = O.out + 5 * N;
    const float* rho = a.m[6];
    const bool pml = !(i >= a.box.i0 && i < a.box.i1 && k >= a.box.k0 && k < a.box.k1);
    const float dt = a.dt;
    const float hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
    const bool ix = inX(i, k, nx, nz), iz = inZ(i, k, nx, nz);
    float vx = O.in[c], vz = O.in[N + c];
    float M8 = 0.f, M11 = 0.f, M10 = 0.f, M9 = 0.f;
    if (ix) {
        const float bxx = inv_mean_f(rho[c], rho[c - 1], a.density_code);
        const float bzx = inv_mean_f(rho[c], rho[c - nx], a.density_code);
        float dsxx_dx = (27.0f * (sxx[c] - sxx[c - 1]) + sxx[c - 2]) * hx;
        float dsxz_dz = (27.0f * (sxz[c] - sxz[c - nx]) + sxz[c - 2 * nx]) * hz;
        if (pml) {
            const float b = a.m[14][c], aa = a.m[12][c], kk = a.m[10][c];
            M8 = b * mi[8 * N + c] + aa * dsxx_dx;
            M11 = b * mi[11 * N + c] + aa * dsxz_dz;
            dsxx_dx = dsxx_dx * kk + M8;
            dsxz_dz = dsxz_dz * kk + M11;
        }
        vx = vx + dt * (dsxx_dx * bxx + dsxz_dz * bzx);
    }
    if (iz) {
        const float bxz = inv_mean_f(rho[c], rho[c + 1], a.density_code);
        const float bzz = inv_mean_f(rho[c], rho[c + nx], a.density_code);
        float dsxz_dx = (27.0f * (sxz[c + 1] - sxz[c]) - sxz[c + 2]) * hx;
        float dszz_dz = (27.0f * (szz[c + nx] - szz[c]) - szz[c + 2 * nx]) * hz;
        if (pml) {
            const float bh = a.m[15][c], ah = a.m[13][c], kh = a.m[11][c];
            M10 = bh * mi[10 * N + c] + ah * dsxz_dx;
            M9 = bh * mi[9 * N + c] + ah * dszz_dz;
            dsxz_dx = dsxz_dx * kh + M10;
            dszz_dz = dszz_dz * kh + M9;
        }
        vz = vz + dt * (dsxz_dx * bxz + dszz_dz * bzz);
    }
    if (i == a.isrc && k == a.jsrc && O.srcz) vz = vz + (float)O.srcz[*O.base + O.j - 1] / rho[c];
    if (i == 0 || i == nx - 1 || k == 0 || k == nz - 1) { vx = 0.f; vz = 0.f; }
    // ---- stores
    if (pml && ix) { mo[8 * N + c] = M8; mo[11 * N + c] = M11; }
    if (pml && iz) { mo[10 * N + c] = M10; mo[9 * N + c] = M9; }
    O.out[c] = vx;
    O.out[N + c] = vz;
}
#undef D4F

// end of a segment: fold its FP32 sums into the FP64 gradient and clear them
__global__ void fold_grad(double* __restrict__ g64, float* __restrict__ g32, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        g64[q] += (double)g32[q];
        g32[q] = 0.0f;
    }
}

}  // namespace

// One shot in flight: its own solver (model copy, fields, stream, graphs),
// checkpoint and segment buffers, adjoint state and FP64 gradient sums.
// Lanes run concurrently on their own streams; their gradients are summed
// on the device at the end.
struct FwiLane {
    SeidartSolver* s = nullptr;
    S2Args<float> a{};          // seismic2 lanes
    E2Args<float> e{};          // electromag2 lanes
    const int* rec = nullptr;
    cudaStream_t st = nullptr;
    StepInfo si{};
    StatePtrs ptrs{};
    int shot = -1;              // shot the lane's solver and graphs are set up for
    bool graphs = false;        // segment graphs captured for `shot`
    float* ckpt = nullptr;      // [G][ns][N]
    float* seg = nullptr;       // [K+1][ns][N]
    float* lam = nullptr;       // [ns][N]
    float* scr = nullptr;       // [12][N]
    float* dres = nullptr;      // [nt][2][nrec] residual of the lane's shot
    double* grad = nullptr;     // [kGradSlots][N] FP64 gradient sums over segments and shots
    float* grad32 = nullptr;    // [kGradSlots][N] FP32 sums within the current segment
    double* dscal = nullptr;    // [0] misfit of the lane's shots
    int* dbase = nullptr;       // device segment base (steps before the segment)
    // [0] full segments of K steps, [1] the shorter last one
    cudaGraphExec_t rec_exec[2] = {nullptr, nullptr}, adj_exec[2] = {nullptr, nullptr};
    long long launches = 0;
};

// gradient accumulator slots per cell: 8 (electromag2: aEx..eEz; seismic2:
// c11 c13 c33 c55 and four face buoyancies) plus c15, c35 for seismic2 with
// the full tensor on
constexpr int kGradSlots = 10;

struct SeidartFwi {
    std::vector<FwiLane> lanes;
    bool full = false;  // seismic2: also dL/dc15, dL/dc35
    int ng() const { return full ? 10 : 8; }  // slots in use
    int family = SEIDART_SEISMIC2, ns = NS;  // solver family and state arrays per cell
    int nrec = 0, nt = 0, nshots = 0, K = 1, G = 1, density = 3;
    size_t N = 0;
    std::vector<int> sx, sz;
    double* dsrc = nullptr;     // [nshots][nt] force series (device)
    float* dobs = nullptr;      // [nshots][nt][2][nrec] observed traces
    double* dgsrc = nullptr;    // [nshots] sum_n lambda(src) f_n per shot (vz or Ez)
    std::vector<double> srch;   // host copy of the source series
    std::vector<double> em[6];  // electromag2: host eps11 eps13 eps33 sig11 sig13 sig33 (for the chain rule)
    int* rfirst = nullptr;      // [N] first receiver at each cell, -1 none (device)
    int* rnext = nullptr;       // [nrec] next receiver at the same cell, -1 none (device)
    double dt = 0.0;
    long long launches = 0;
};

namespace {
std::string g_ferr;
int ferr(int code, const std::string& m) {
    g_ferr = m;
    return code;
}
#define FCUDA(x)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (x);                                                      \
        if (e_ != cudaSuccess) return ferr(SEIDART_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

// sum of lane gradients: dst[q] += src[q]
__global__ void add_grad(double* __restrict__ dst, const double* __restrict__ src, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        dst[q] += src[q];
}

AdjArgs adj_args(SeidartFwi* f, FwiLane& L, const float* xp, const float* xc, const double* srcz, int j) {
    AdjArgs A{};
    A.nx = L.a.nx; A.nz = L.a.nz; A.density_code = L.a.density_code;
    A.dt = L.a.dt; A.hx = 1.0f / (24.0f * L.a.dx); A.hz = 1.0f / (24.0f * L.a.dz);
    A.box = L.a.box;
    for (int q = 0; q < 16; ++q) A.m[q] = L.a.m[q];
    A.xp = xp; A.xc = xc; A.lam = L.lam; A.scr = L.scr; A.grad = L.grad32; A.N = f->N;
    A.isrc = L.a.isrc; A.jsrc = L.a.jsrc; A.srcz = srcz;
    A.gsrc = f->dgsrc + (L.shot >= 0 ? L.shot : 0);
    A.base = L.dbase; A.j = j;
    A.rfirst = f->rfirst; A.rnext = f->rnext; A.nrec = f->nrec;
    A.dres = f->nrec > 0 ? L.dres : nullptr;
    A.full = f->full ? 1 : 0;
    return A;
}

EmAdjArgs em_args(SeidartFwi* f, FwiLane& L, const float* xp, const float* xc, const double* srcz, int j) {
    EmAdjArgs A{};
    A.a = L.e;
    A.xp = xp; A.xc = xc; A.lam = L.lam; A.scr = L.scr; A.grad = L.grad32; A.N = f->N;
    A.srcz = srcz; A.base = L.dbase; A.j = j;
    A.gsrc = f->dgsrc + (L.shot >= 0 ? L.shot : 0);
    A.rfirst = f->rfirst; A.rnext = f->rnext; A.nrec = f->nrec;
    A.dres = f->nrec > 0 ? L.dres : nullptr;
    return A;
}

// grid extent of the lane's solver
int lane_nx(const SeidartFwi* f, const FwiLane& L) { return f->family == SEIDART_ELECTROMAG2 ? L.e.nx : L.a.nx; }
int lane_nz(const SeidartFwi* f, const FwiLane& L) { return f->family == SEIDART_ELECTROMAG2 ? L.e.nz : L.a.nz; }
float* lane_traces(const SeidartFwi* f, const FwiLane& L) {
    return f->family == SEIDART_ELECTROMAG2 ? L.e.traces : L.a.traces;
}
double* lane_norms(const SeidartFwi* f, const FwiLane& L) {
    return f->family == SEIDART_ELECTROMAG2 ? L.e.norms : L.a.norms;
}

// Adjoint of step n = *dbase + j (launched on the lane's stream, possibly
// under capture): two grid passes.  The receiver residuals of step n
// (inject = false: none) are added by the first pass, which also finishes the
// gather left by step n+1; the gather this step leaves is finished by step
// n-1 (or by adjoint_flush).
void adjoint_step(SeidartFwi* f, FwiLane& L, int j, const float* xp, const float* xc, const double* srcz,
                  bool inject) {
    if (f->family == SEIDART_ELECTROMAG2) {
        EmAdjArgs A = em_args(f, L, xp, xc, srcz, j);
        if (!inject) A.dres = nullptr;
        em2_adjoint_step(A, L.st);
        return;
    }
    const dim3 blk(BX, BY), grd((L.a.nx + BX - 1) / BX, (L.a.nz + BY - 1) / BY);
    AdjArgs A = adj_args(f, L, xp, xc, srcz, j);
    if (!inject) A.dres = nullptr;
    adj_velocity<<<grd, blk, 0, L.st>>>(A);
    adj_stress<<<grd, blk, 0, L.st>>>(A);
}

void adjoint_flush(SeidartFwi* f, FwiLane& L, const float* xp, const float* xc) {
    if (f->family == SEIDART_ELECTROMAG2) {
        em2_adjoint_flush(em_args(f, L, xp, xc, nullptr, 1), L.st);
        return;
    }
    const dim3 blk(BX, BY), grd((L.a.nx + BX - 1) / BX, (L.a.nz + BY - 1) / BY);
    adj_flush_v<<<grd, blk, 0, L.st>>>(adj_args(f, L, xp, xc, nullptr, 1));
}

void save_state(const SeidartFwi* f, FwiLane& L, float* blk) {
    copy_state<<<4 * 152, 256, 0, L.st>>>(L.ptrs, blk, f->N, 1, f->ns);
    ++L.launches;
}
void load_state(const SeidartFwi* f, FwiLane& L, const float* blk) {
    copy_state<<<4 * 152, 256, 0, L.st>>>(L.ptrs, const_cast<float*>(blk), f->N, 0, f->ns);
    ++L.launches;
}

// refresh the lane's copy of its solver's FP32 arguments
void lane_args(SeidartFwi* f, FwiLane& L, const int** rec) {
    if (f->family == SEIDART_ELECTROMAG2) seidart_solver_internal_e2f(L.s, &L.e, rec);
    else seidart_solver_internal_s2f(L.s, &L.a, rec);
}

// Point lane L at shot sh (its source position and series).  Waits for the
// lane's stream only when the shot changes.
int lane_set_shot(SeidartFwi* f, FwiLane& L, int sh) {
    if (L.shot == sh) return SEIDART_OK;
    const int rc = seidart_solver_internal_set_source(L.s, f->sx[sh], f->sz[sh], nullptr, f->dsrc + (size_t)sh * f->nt);
    if (rc != SEIDART_OK) return ferr(rc, seidart_last_error());
    lane_args(f, L, nullptr);
    L.shot = sh;
    L.graphs = false;
    return SEIDART_OK;
}

// zero the lane's state, traces and norms and restart its step counter,
// all queued on the lane's stream (no host wait)
int lane_reset(SeidartFwi* f, FwiLane& L) {
    const size_t N = f->N;
    for (int q = 0; q < f->ns; ++q) FCUDA(cudaMemsetAsync(L.ptrs.p[q], 0, sizeof(float) * N, L.st));
    FCUDA(cudaMemsetAsync(lane_traces(f, L), 0, sizeof(float) * (size_t)f->nt * 2 * (f->nrec > 0 ? f->nrec : 1), L.st));
    FCUDA(cudaMemsetAsync(lane_norms(f, L), 0, sizeof(double) * f->nt, L.st));
    seg_begin<<<1, 1, 0, L.st>>>(L.si.step, L.dbase, 0);
    FCUDA(cudaGetLastError());
    seidart_solver_internal_advance(L.s, -seidart_solver_steps_done(L.s));
    return SEIDART_OK;
}

// forward segment g of lane L (checkpoint first when asked)
int lane_forward_segment(SeidartFwi* f, FwiLane& L, int g, bool checkpoints) {
    const int t0 = g * f->K, len = std::min(f->K, f->nt - t0);
    if (checkpoints) save_state(f, L, L.ckpt + (size_t)g * f->ns * f->N);
    const int rc = seidart_solver_step(L.s, len);
    if (rc != SEIDART_OK) return ferr(rc, seidart_last_error());
    L.launches += (long long)len * seidart_step_launches(f->family, f->family == SEIDART_SEISMIC2 ? L.a.stress_src : 0);
    return SEIDART_OK;
}

int lane_residual(SeidartFwi* f, FwiLane& L) {
    const size_t n = (size_t)f->nt * 2 * f->nrec;
    if (n == 0) return SEIDART_OK;
    residual_loss<<<152, 256, 0, L.st>>>(lane_traces(f, L), f->dobs + (size_t)L.shot * n, L.dres, n, L.dscal);
    ++L.launches;
    return cudaGetLastError() == cudaSuccess ? SEIDART_OK : ferr(SEIDART_ERR_CUDA, "residual kernel");
}

// Capture the recompute graph (len forward steps, each state saved to the
// segment buffer) or the adjoint graph (len adjoint steps, last to first)
// and instantiate it into *exec, updating an existing executable in place
// when the topology allows.
int capture_segment(SeidartFwi* f, FwiLane& L, int len, bool adjoint, cudaGraphExec_t* exec) {
    const size_t state = (size_t)f->ns * f->N;
    const double* srcz = f->dsrc + (size_t)L.shot * f->nt;
    FCUDA(cudaStreamBeginCapture(L.st, cudaStreamCaptureModeThreadLocal));
    const dim3 blk(BX, BY), grd((L.a.nx + BX - 1) / BX, (L.a.nz + BY - 1) / BY);
    if (!adjoint && f->family == SEIDART_ELECTROMAG2) {
        for (int j = 1; j <= len; ++j) {
            const EmOopArgs O{L.e, L.seg + (size_t)(j - 1) * state, L.seg + (size_t)j * state, f->N, srcz, L.dbase, j};
            em2_recompute_step(O, L.st);
        }
    } else if (!adjoint) {
        for (int j = 1; j <= len; ++j) {
            OopArgs O{L.a, L.seg + (size_t)(j - 1) * state, L.seg + (size_t)j * state, f->N, srcz, L.dbase, j};
            oop_stress<<<grd, blk, 0, L.st>>>(O);
            oop_velocity<<<grd, blk, 0, L.st>>>(O);
        }
    } else {
        for (int j = len; j >= 1; --j)
            adjoint_step(f, L, j, L.seg + (size_t)(j - 1) * state, L.seg + (size_t)j * state, srcz, true);
        fold_grad<<<4 * 152, 256, 0, L.st>>>(L.grad, L.grad32, (size_t)f->ng() * f->N);
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(L.st, &g);
    if (e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        return ferr(SEIDART_ERR_CUDA, std::string("segment capture: ") + cudaGetErrorString(e));
    }
    if (*exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(*exec, g, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(*exec);
            *exec = nullptr;
        }
    }
    if (!*exec) e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return ferr(SEIDART_ERR_CUDA, std::string("segment graph: ") + cudaGetErrorString(e));
    return SEIDART_OK;
}

int lane_graphs(SeidartFwi* f, FwiLane& L) {
    if (L.graphs) return SEIDART_OK;
    const int last = f->nt - (f->G - 1) * f->K;  // length of the last segment
    const int lens[2] = {f->K, last};
    for (int slot = 0; slot < 2; ++slot) {
        if (slot == 1 && last == f->K) break;
        int rc = capture_segment(f, L, lens[slot], false, &L.rec_exec[slot]);
        if (rc == SEIDART_OK) rc = capture_segment(f, L, lens[slot], true, &L.adj_exec[slot]);
        if (rc != SEIDART_OK) return rc;
    }
    L.graphs = true;
    return SEIDART_OK;
}

// adjoint segment g of lane L: restore the checkpoint, recompute, walk back
int lane_backward_segment(SeidartFwi* f, FwiLane& L, int g) {
    const int t0 = g * f->K, len = std::min(f->K, f->nt - t0);
    const int slot = len == f->K ? 0 : 1;
    seg_begin<<<1, 1, 0, L.st>>>(L.si.step, L.dbase, t0);
    FCUDA(cudaMemcpyAsync(L.seg, L.ckpt + (size_t)g * f->ns * f->N, sizeof(float) * f->ns * f->N,
                          cudaMemcpyDeviceToDevice, L.st));
    FCUDA(cudaGetLastError());
    FCUDA(cudaGraphLaunch(L.rec_exec[slot], L.st));
    FCUDA(cudaGraphLaunch(L.adj_exec[slot], L.st));
    L.launches += 1 + 2 * len + 2 * len + 1;
    return SEIDART_OK;
}

// Run every shot: forward (with checkpoints when grad), misfit, and when grad
// the adjoint sweep.  Shots go to lanes in rounds of nlanes; within a round
// the host queues segment by segment across lanes so their streams overlap.
int run_shots(SeidartFwi* f, bool grad, bool keep_traces_of_round, double* traces_out) {
    const int nl = (int)f->lanes.size();
    const size_t ntr = (size_t)f->nt * 2 * f->nrec;
    for (int r0 = 0; r0 < f->nshots; r0 += nl) {
        const int nr = std::min(nl, f->nshots - r0);
        for (int l = 0; l < nr; ++l) {
            int rc = lane_set_shot(f, f->lanes[l], r0 + l);
            if (rc == SEIDART_OK) rc = lane_reset(f, f->lanes[l]);
            if (rc != SEIDART_OK) return rc;
        }
        for (int g = 0; g < f->G; ++g)
            for (int l = 0; l < nr; ++l) {
                const int rc = lane_forward_segment(f, f->lanes[l], g, grad);
                if (rc != SEIDART_OK) return rc;
            }
        for (int l = 0; l < nr; ++l) {
            FwiLane& L = f->lanes[l];
            const int rc = lane_residual(f, L);
            if (rc != SEIDART_OK) return rc;
            if (keep_traces_of_round) {
                int rc2 = seidart_solver_sync(L.s);
                if (rc2 == SEIDART_OK) rc2 = seidart_solver_traces(L.s, traces_out + (size_t)L.shot * ntr, nullptr);
                if (rc2 != SEIDART_OK) return ferr(rc2, seidart_last_error());
            }
        }
        if (!grad) continue;
        for (int l = 0; l < nr; ++l) {
            FwiLane& L = f->lanes[l];
            FCUDA(cudaMemsetAsync(L.lam, 0, sizeof(float) * f->ns * f->N, L.st));
            FCUDA(cudaMemsetAsync(L.scr, 0, sizeof(float) * 12 * f->N, L.st));
            const int rc = lane_graphs(f, L);
            if (rc != SEIDART_OK) return rc;
        }
        for (int g = f->G - 1; g >= 0; --g)
            for (int l = 0; l < nr; ++l) {
                const int rc = lane_backward_segment(f, f->lanes[l], g);
                if (rc != SEIDART_OK) return rc;
            }
    }
    return SEIDART_OK;
}

int sync_lanes(SeidartFwi* f) {
    for (auto& L : f->lanes) {
        const int rc = seidart_solver_sync(L.s);
        if (rc != SEIDART_OK) return ferr(rc, seidart_last_error());
    }
    return SEIDART_OK;
}

size_t lane_bytes(size_t N, int ns, int K, int G, int nt, int nrec) {
    return sizeof(float) * ((size_t)G + K + 1 + 1 + 0) * ns * N + sizeof(float) * 12 * N +
           (sizeof(double) + sizeof(float)) * kGradSlots * N +
           sizeof(float) * (size_t)nt * 2 * (nrec > 0 ? nrec : 1) + sizeof(float) * 40 * N;  // + solver arena
}

void free_lane(FwiLane& L) {
    if (L.st) cudaStreamSynchronize(L.st);
    for (int q = 0; q < 2; ++q) {
        if (L.rec_exec[q]) cudaGraphExecDestroy(L.rec_exec[q]);
        if (L.adj_exec[q]) cudaGraphExecDestroy(L.adj_exec[q]);
    }
    for (void* p : {(void*)L.ckpt, (void*)L.seg, (void*)L.lam, (void*)L.scr, (void*)L.dres, (void*)L.grad,
                    (void*)L.grad32, (void*)L.dscal, (void*)L.dbase})
        if (p) cudaFree(p);
    if (L.s) seidart_solver_destroy(L.s);
    L = FwiLane();
}

// Chain dL/d(aEx bEx dEx eEx aEz bEz dEz eEz) per cell to the relative
// permittivities and conductivities (cpmlfdtd.f08:2519-2540: eps scaled by
// eps0, det = eps11 eps33 - eps13^2 clamped at 1e-18 eps0^2, where its
// derivative is zero), plus the Ez source term f dt / eps33 at each shot's
// cell.  out: [6][N] eps11 eps13 eps33 sig11 sig13 sig33.
void em_chain(const SeidartFwi* f, const std::vector<double>& g, const std::vector<double>& gsrc, double* out) {
    const size_t N = f->N;
    const double eps0 = 8.85418782e-12;  // constants.f08
    const double floor = 1.0e-18 * eps0 * eps0;
    for (size_t q = 0; q < N; ++q) {
        const double E11 = f->em[0][q] * eps0, E13 = f->em[1][q] * eps0, E33 = f->em[2][q] * eps0;
        const double s11 = f->em[3][q], s13 = f->em[4][q], s33 = f->em[5][q];
        double det = E11 * E33 - E13 * E13;
        double dd[6] = {E33, -2.0 * E13, E11, 0.0, 0.0, 0.0};
        if (det <= floor) {
            det = floor;
            for (double& v : dd) v = 0.0;
        }
        // numerators of the eight coefficients and their partials in (E11 E13 E33 s11 s13 s33)
        const double num[8] = {E33, -E13, E33 * s11 - E13 * s13, E33 * s13 - E13 * s33,
                               -E13, E11, E11 * s13 - E13 * s11, E11 * s33 - E13 * s13};
        const double dn[8][6] = {{0, 0, 1, 0, 0, 0},         {0, -1, 0, 0, 0, 0},
                                 {0, -s13, s11, E33, -E13, 0}, {0, -s33, s13, 0, E33, -E13},
                                 {0, -1, 0, 0, 0, 0},         {1, 0, 0, 0, 0, 0},
                                 {s13, -s11, 0, -E13, E11, 0}, {s33, -s13, 0, 0, -E13, E11}};
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int w = 0; w < 8; ++w) {
            const double gw = g[(size_t)w * N + q];
            if (gw == 0.0) continue;
            const double coef = num[w] / det;
            for (int p = 0; p < 6; ++p) acc[p] += gw * (dn[w][p] - coef * dd[p]) / det;
        }
        for (int p = 0; p < 3; ++p) out[(size_t)p * N + q] = acc[p] * eps0;
        for (int p = 3; p < 6; ++p) out[(size_t)p * N + q] = acc[p];
    }
    for (int sh = 0; sh < f->nshots; ++sh) {
        const size_t c = (size_t)f->sx[sh] + (size_t)lane_nx(f, f->lanes[0]) * f->sz[sh];
        const double E33 = f->em[2][c] * eps0;
        out[2 * N + c] += -gsrc[sh] * f->dt / (E33 * E33) * eps0;
    }
}

}  // namespace

extern "C" {

const char* seidart_fwi_last_error(void) { return g_ferr.c_str(); }

int seidart_fwi_destroy(SeidartFwi* f) {
    if (!f) return SEIDART_OK;
    for (auto& L : f->lanes) free_lane(L);
    for (void* p : {(void*)f->dsrc, (void*)f->dobs, (void*)f->dgsrc, (void*)f->rfirst, (void*)f->rnext})
        if (p) cudaFree(p);
    delete f;
    return SEIDART_OK;
}

// Create an FWI problem: one 2D model (host FP64, the family's slots), shots
// with their own source position (interior indices) and source series (the
// vertical force of seismic2, the Ez source of electromag2), a common
// receiver set, and observed traces per shot ([time_steps][2][nrec]: vx, vz
// or Ex, Ez).  checkpoint_every = 0 picks ceil(sqrt(nt)).  Up to one lane
// per shot, as device memory allows.
int seidart_fwi_create_family(SeidartFwi** out, int family, const SeidartDomain* dom, const SeidartSource* src,
                              int density_code, const double* const* model, int nshots, const int* shot_xind,
                              const int* shot_zind, const double* const* shot_srcz, int nrec, const int* rec_cells,
                              const double* const* observed, int checkpoint_every) {
    seidart_trace::Range nvtx("seidart_fwi_create");
    if (!out || !dom || !src || !model || nshots < 1 || !shot_xind || !shot_zind || !shot_srcz)
        return ferr(SEIDART_ERR_ARG, "bad arguments");
    if (family != SEIDART_SEISMIC2 && family != SEIDART_ELECTROMAG2)
        return ferr(SEIDART_ERR_UNSUPPORTED, "the adjoint covers seismic2 and electromag2");
    *out = nullptr;
    SeidartFwi* f = new SeidartFwi();
    f->family = family;
    f->ns = family == SEIDART_ELECTROMAG2 ? NS_EM : NS;
    f->dt = src->dt;
    f->nt = src->time_steps;
    f->nshots = nshots;
    f->nrec = nrec;
    f->density = density_code;
    f->N = (size_t)dom->nx * dom->nz;
    if (family == SEIDART_ELECTROMAG2)
        for (int q = 0; q < 6; ++q) f->em[q].assign(model[E2_E11 + q], model[E2_E11 + q] + f->N);
    f->K = checkpoint_every > 0 ? checkpoint_every : (int)ceil(sqrt((double)f->nt));
    f->G = (f->nt + f->K - 1) / f->K;
    for (int sh = 0; sh < nshots; ++sh) {
        f->sx.push_back(shot_xind[sh] + dom->cpml - 1);
        f->sz.push_back(shot_zind[sh] + dom->cpml - 1);
        if (f->sx.back() < 0 || f->sx.back() + 1 >= dom->nx || f->sz.back() < 0 || f->sz.back() + 1 >= dom->nz) {
            seidart_fwi_destroy(f);
            return ferr(SEIDART_ERR_ARG, "shot source outside the grid");
        }
        f->srch.insert(f->srch.end(), shot_srcz[sh], shot_srcz[sh] + f->nt);
    }
    const size_t nobs = (size_t)f->nt * 2 * nrec;
    if (cudaMalloc((void**)&f->dsrc, sizeof(double) * nshots * f->nt) != cudaSuccess ||
        cudaMalloc((void**)&f->dobs, sizeof(float) * nshots * (nobs ? nobs : 1)) != cudaSuccess ||
        cudaMalloc((void**)&f->dgsrc, sizeof(double) * nshots) != cudaSuccess) {
        cudaGetLastError();
        seidart_fwi_destroy(f);
        return ferr(SEIDART_ERR_NOMEM, "FWI buffer allocation failed");
    }
    // a failed upload of the sources, receiver chains or observed traces
    // ends the set-up with the CUDA error
    auto upload_failed = [&]() {
        const std::string m = std::string("FWI upload failed: ") + cudaGetErrorString(cudaGetLastError());
        seidart_fwi_destroy(f);
        return ferr(SEIDART_ERR_CUDA, m);
    };
    if (cudaMemcpy(f->dsrc, f->srch.data(), sizeof(double) * nshots * f->nt, cudaMemcpyHostToDevice) != cudaSuccess)
        return upload_failed();
    {   // receiver chains per cell (several receivers may share a cell)
        std::vector<int> first(f->N, -1), next(nrec > 0 ? nrec : 1, -1);
        for (int r = nrec - 1; r >= 0; --r) {
            const int c = rec_cells[r];
            if (c < 0 || (size_t)c >= f->N) {
                seidart_fwi_destroy(f);
                return ferr(SEIDART_ERR_ARG, "receiver cell outside the grid");
            }
            next[r] = first[c];
            first[c] = r;
        }
        if (cudaMalloc((void**)&f->rfirst, sizeof(int) * f->N) != cudaSuccess ||
            cudaMalloc((void**)&f->rnext, sizeof(int) * next.size()) != cudaSuccess) {
            cudaGetLastError();
            seidart_fwi_destroy(f);
            return ferr(SEIDART_ERR_NOMEM, "FWI buffer allocation failed");
        }
        if (cudaMemcpy(f->rfirst, first.data(), sizeof(int) * f->N, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(f->rnext, next.data(), sizeof(int) * next.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return upload_failed();
    }
    std::vector<float> tmp(nobs);
    for (int sh = 0; sh < nshots && nobs; ++sh) {
        if (!observed || !observed[sh]) {
            std::fill(tmp.begin(), tmp.end(), 0.f);
        } else {
            for (size_t q = 0; q < nobs; ++q) tmp[q] = (float)observed[sh][q];
        }
        if (cudaMemcpy(f->dobs + (size_t)sh * nobs, tmp.data(), sizeof(float) * nobs, cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return upload_failed();
    }
    // lanes: enough concurrent shots for about 1.2 M cells in flight (on a
    // 552^2 grid 4 lanes measured 2.57 s per 16-shot gradient, 16 lanes
    // 2.75 s, 1 lane 3.81 s), within 3/4 of the free device memory
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t per = lane_bytes(f->N, f->ns, f->K, f->G, f->nt, nrec);
    // (SEIDART_FWI_LANES sets the number instead, within the shots and memory)
    size_t want = std::max<size_t>(1, (size_t)(1.2e6 / (double)f->N + 0.5));
    const char* env = getenv("SEIDART_FWI_LANES");
    if (env && atoi(env) > 0) want = (size_t)atoi(env);
    const int nl = (int)std::min<size_t>(std::min<size_t>((size_t)nshots, want), std::max<size_t>(1, (free_b / 4 * 3) / per));
    f->lanes.resize(nl);
    for (int l = 0; l < nl; ++l) {
        FwiLane& L = f->lanes[l];
        // the force (seismic2) or the Ez source (electromag2) is the second source slot
        const double* srcs[S2_NSRC] = {nullptr, shot_srcz[l], nullptr, nullptr, nullptr};
        SeidartSource s0 = *src;
        s0.xind = shot_xind[l];
        s0.zind = shot_zind[l];
        int rc = seidart_solver_create(&L.s, family, SEIDART_FP32, dom, &s0, density_code, model, srcs, nrec,
                                       rec_cells);
        // every shot runs on one model: the lanes read lane 0's copy, so the
        // concurrent shots keep one model in L2 instead of one each
        if (rc == SEIDART_OK && l > 0) rc = seidart_solver_internal_share_model(L.s, f->lanes[0].s);
        if (rc != SEIDART_OK) { std::string e = seidart_last_error(); seidart_fwi_destroy(f); return ferr(rc, e); }
        lane_args(f, L, &L.rec);
        L.st = seidart_solver_internal_stream(L.s);
        L.si = seidart_solver_internal_stepinfo(L.s);
        if (family == SEIDART_ELECTROMAG2) {
            for (int q = 0; q < 3; ++q) L.ptrs.p[q] = L.e.f[q];
            for (int q = 0; q < 4; ++q) L.ptrs.p[3 + q] = L.e.mem[q];
        } else {
            for (int q = 0; q < 5; ++q) L.ptrs.p[q] = L.a.f[q];
            for (int q = 0; q < 12; ++q) L.ptrs.p[5 + q] = L.a.mem[q];
        }
        if (cudaMalloc((void**)&L.ckpt, sizeof(float) * f->G * f->ns * f->N) != cudaSuccess ||
            cudaMalloc((void**)&L.seg, sizeof(float) * (f->K + 1) * f->ns * f->N) != cudaSuccess ||
            cudaMalloc((void**)&L.lam, sizeof(float) * f->ns * f->N) != cudaSuccess ||
            cudaMalloc((void**)&L.scr, sizeof(float) * 12 * f->N) != cudaSuccess ||
            cudaMalloc((void**)&L.dres, sizeof(float) * (nobs ? nobs : 1)) != cudaSuccess ||
            cudaMalloc((void**)&L.grad, sizeof(double) * kGradSlots * f->N) != cudaSuccess ||
            cudaMalloc((void**)&L.grad32, sizeof(float) * kGradSlots * f->N) != cudaSuccess ||
            cudaMalloc((void**)&L.dscal, sizeof(double) * 2) != cudaSuccess ||
            cudaMalloc((void**)&L.dbase, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            seidart_fwi_destroy(f);
            return ferr(SEIDART_ERR_NOMEM, "FWI lane allocation failed");
        }
        // segment states are written only where a step updates them: start from zeros
        if (cudaMemset(L.seg, 0, sizeof(float) * (f->K + 1) * f->ns * f->N) != cudaSuccess ||
            cudaMemset(L.grad32, 0, sizeof(float) * kGradSlots * f->N) != cudaSuccess) {
            cudaGetLastError();
            seidart_fwi_destroy(f);
            return ferr(SEIDART_ERR_CUDA, "FWI lane initialisation failed");
        }
        // the solver was created with shot l's source: point the lane at the shared series
        rc = lane_set_shot(f, L, l);
        if (rc != SEIDART_OK) { seidart_fwi_destroy(f); return rc; }
    }
    *out = f;
    return SEIDART_OK;
}

int seidart_fwi_create(SeidartFwi** out, const SeidartDomain* dom, const SeidartSource* src, int density_code,
                       const double* const* model, int nshots, const int* shot_xind, const int* shot_zind,
                       const double* const* shot_srcz, int nrec, const int* rec_cells,
                       const double* const* observed, int checkpoint_every) {
    return seidart_fwi_create_family(out, SEIDART_SEISMIC2, dom, src, density_code, model, nshots, shot_xind,
                                     shot_zind, shot_srcz, nrec, rec_cells, observed, checkpoint_every);
}

// Loss and gradient over all shots.  grad (host, may be NULL) receives FP64
// per cell: seismic2 [5][ncell] dL/dc11, dL/dc13, dL/dc33, dL/dc55, dL/drho
// (and [7][ncell] with dL/dc15, dL/dc35 after them when the full tensor is on);
// electromag2 [6][ncell] dL/deps11, dL/deps13, dL/deps33 (relative
// permittivities, as in e11.dat ...), dL/dsig11, dL/dsig13, dL/dsig33.
int seidart_fwi_gradient(SeidartFwi* f, double* loss, double* grad) {
    seidart_trace::Range nvtx("seidart_fwi_gradient");
    if (!f) return ferr(SEIDART_ERR_ARG, "NULL");
    f->launches = 0;
    for (auto& L : f->lanes) {
        L.launches = 0;
        FCUDA(cudaMemsetAsync(L.grad, 0, sizeof(double) * kGradSlots * f->N, L.st));
        FCUDA(cudaMemsetAsync(L.grad32, 0, sizeof(float) * kGradSlots * f->N, L.st));
        FCUDA(cudaMemsetAsync(L.dscal, 0, sizeof(double) * 2, L.st));
    }
    FCUDA(cudaMemsetAsync(f->dgsrc, 0, sizeof(double) * f->nshots, f->lanes[0].st));
    FCUDA(cudaStreamSynchronize(f->lanes[0].st));
    int rc = run_shots(f, grad != nullptr, false, nullptr);
    if (rc != SEIDART_OK) return rc;
    rc = sync_lanes(f);
    if (rc != SEIDART_OK) return rc;
    double total = 0.0;
    for (auto& L : f->lanes) {
        double l = 0.0;
        FCUDA(cudaMemcpy(&l, L.dscal, sizeof(double), cudaMemcpyDeviceToHost));
        total += l;
        f->launches += L.launches;
    }
    if (loss) *loss = total;
    if (grad) {
        const size_t N = f->N;
        FwiLane& L0 = f->lanes[0];
        for (size_t l = 1; l < f->lanes.size(); ++l) {
            add_grad<<<4 * 152, 256, 0, L0.st>>>(L0.grad, f->lanes[l].grad, (size_t)f->ng() * N);
            ++f->launches;
        }
        FCUDA(cudaGetLastError());
        FCUDA(cudaStreamSynchronize(L0.st));
        std::vector<double> g((size_t)f->ng() * N), gsrc(f->nshots);
        FCUDA(cudaMemcpy(g.data(), L0.grad, sizeof(double) * f->ng() * N, cudaMemcpyDeviceToHost));
        FCUDA(cudaMemcpy(gsrc.data(), f->dgsrc, sizeof(double) * f->nshots, cudaMemcpyDeviceToHost));
        if (f->family == SEIDART_ELECTROMAG2) {
            em_chain(f, g, gsrc, grad);
            return SEIDART_OK;
        }
        memcpy(grad, g.data(), sizeof(double) * 4 * N);
        if (f->full) memcpy(grad + 5 * N, g.data() + 8 * N, sizeof(double) * 2 * N);  // c15, c35 after rho
        // chain the face buoyancies B = 1/mean(rho_a, rho_b) to rho (FP32 forward values)
        std::vector<float> rho(N);
        FCUDA(cudaMemcpy(rho.data(), L0.a.m[S2_RHO], sizeof(float) * N, cudaMemcpyDeviceToHost));
        double* gr = grad + 4 * N;
        for (size_t q = 0; q < N; ++q) gr[q] = 0.0;
        const int nx = L0.a.nx, code = f->density;
        auto dB = [code](double a, double b, double* da, double* db) {
            switch (code) {
            case 1: *da = -1.0 / (2.0 * a * a); *db = -1.0 / (2.0 * b * b); break;       // (a+b)/(2ab)
            case 2: { const double B = 1.0 / sqrt(a * b); *da = -B / (2.0 * a); *db = -B / (2.0 * b); break; }
            case 3: { const double s = a + b; *da = *db = -2.0 / (s * s); break; }       // 2/(a+b)
            default: *da = -1.0 / (a * a); *db = 0.0; break;                            // 1/a
            }
        };
        const size_t sz = (size_t)nx;
        for (size_t q = 0; q < N; ++q) {
            double da, db;
            if (g[4 * N + q] != 0.0) { dB(rho[q], rho[q - 1], &da, &db); gr[q] += g[4 * N + q] * da; gr[q - 1] += g[4 * N + q] * db; }
            if (g[5 * N + q] != 0.0) { dB(rho[q], rho[q - sz], &da, &db); gr[q] += g[5 * N + q] * da; gr[q - sz] += g[5 * N + q] * db; }
            if (g[6 * N + q] != 0.0) { dB(rho[q], rho[q + 1], &da, &db); gr[q] += g[6 * N + q] * da; gr[q + 1] += g[6 * N + q] * db; }
            if (g[7 * N + q] != 0.0) { dB(rho[q], rho[q + sz], &da, &db); gr[q] += g[7 * N + q] * da; gr[q + sz] += g[7 * N + q] * db; }
        }
        // force source term vz(src) += f_n / rho(src)
        for (int sh = 0; sh < f->nshots; ++sh) {
            const size_t c = (size_t)f->sx[sh] + sz * f->sz[sh];
            gr[c] += -gsrc[sh] / ((double)rho[c] * (double)rho[c]);
        }
    }
    return SEIDART_OK;
}

// Synthetic traces of every shot for the current model ([nshots][nt][2][nrec]).
int seidart_fwi_model_traces(SeidartFwi* f, double* traces) {
    if (!f || !traces) return ferr(SEIDART_ERR_ARG, "NULL");
    for (auto& L : f->lanes) FCUDA(cudaMemsetAsync(L.dscal, 0, sizeof(double) * 2, L.st));
    int rc = run_shots(f, false, true, traces);
    if (rc == SEIDART_OK) rc = sync_lanes(f);
    return rc;
}

// Adjoint test hook: apply one adjoint step (no receiver residual) to the
// adjoint state lam (host, [ns][ncell] FP32 in state order: 17 arrays for
// seismic2, 7 for electromag2) with forward states xprev/xcur
// ([ns][ncell]); lam is updated in place.
int seidart_fwi_adjoint_step_host(SeidartFwi* f, const float* xprev, const float* xcur, float* lam) {
    if (!f || !xprev || !xcur || !lam) return ferr(SEIDART_ERR_ARG, "NULL");
    FwiLane& L = f->lanes[0];
    const size_t bytes = sizeof(float) * f->ns * f->N;
    float *dp = nullptr, *dc = nullptr;
    FCUDA(cudaMalloc((void**)&dp, bytes));
    FCUDA(cudaMalloc((void**)&dc, bytes));
    FCUDA(cudaMemcpy(dp, xprev, bytes, cudaMemcpyHostToDevice));
    FCUDA(cudaMemcpy(dc, xcur, bytes, cudaMemcpyHostToDevice));
    FCUDA(cudaMemcpy(L.lam, lam, bytes, cudaMemcpyHostToDevice));
    FCUDA(cudaMemsetAsync(L.dbase, 0, sizeof(int), L.st));
    FCUDA(cudaMemsetAsync(L.scr, 0, sizeof(float) * 12 * f->N, L.st));
    adjoint_step(f, L, 1, dp, dc, nullptr, false);
    // the step leaves its last gather to the next step: finish it here
    adjoint_flush(f, L, dp, dc);
    FCUDA(cudaGetLastError());
    FCUDA(cudaStreamSynchronize(L.st));
    FCUDA(cudaMemcpy(lam, L.lam, bytes, cudaMemcpyDeviceToHost));
    cudaFree(dp);
    cudaFree(dc);
    return SEIDART_OK;
}

// Forward test hook: one forward step (source off) on a host state [ns][ncell].
int seidart_fwi_forward_step_host(SeidartFwi* f, float* x) {
    if (!f || !x) return ferr(SEIDART_ERR_ARG, "NULL");
    FwiLane& L = f->lanes[0];
    const size_t bytes = sizeof(float) * f->ns * f->N;
    float* d = nullptr;
    FCUDA(cudaMalloc((void**)&d, bytes));
    FCUDA(cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice));
    int rc = seidart_solver_internal_reset(L.s);
    if (rc == SEIDART_OK) rc = seidart_solver_internal_set_source(L.s, f->sx[0], f->sz[0], nullptr, nullptr);
    if (rc == SEIDART_OK) {
        lane_args(f, L, nullptr);
        load_state(f, L, d);
        rc = seidart_solver_step(L.s, 1);
    }
    if (rc == SEIDART_OK) save_state(f, L, d);
    FCUDA(cudaStreamSynchronize(L.st));
    FCUDA(cudaMemcpy(x, d, bytes, cudaMemcpyDeviceToHost));
    cudaFree(d);
    // the lane's source was switched off: set it up again before the next run
    L.shot = -1;
    const int rc2 = lane_set_shot(f, L, 0);
    if (rc != SEIDART_OK) return ferr(rc, seidart_last_error());
    return rc2;
}

long long seidart_fwi_launches(const SeidartFwi* f) { return f ? f->launches : -1; }

int seidart_fwi_set_full_tensor(SeidartFwi* f, int on) {
    if (!f) return ferr(SEIDART_ERR_ARG, "NULL");
    if (f->family != SEIDART_SEISMIC2) return ferr(SEIDART_ERR_ARG, "the full-tensor gradient is for seismic2");
    if (f->full != (on != 0)) {
        f->full = on != 0;
        // the flag is baked into the captured segment graphs: capture again
        for (auto& L : f->lanes) {
            FCUDA(cudaStreamSynchronize(L.st));
            L.graphs = false;
        }
    }
    return SEIDART_OK;
}
int seidart_fwi_checkpointing(const SeidartFwi* f, int* every, int* count) {
    if (!f) return ferr(SEIDART_ERR_ARG, "NULL");
    if (every) *every = f->K;
    if (count) *count = f->G;
    return SEIDART_OK;
}

}  // extern "C"
