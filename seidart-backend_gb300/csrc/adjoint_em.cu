// adjoint_em.cu -- discrete adjoint of one FP32 step of the 2D
// electromagnetic solver (electromag2, src/fortran/cpmlfdtd.f08:2566-2748),
// and the out-of-place forward step the checkpointed sweep recomputes with.
//
// State x = (Ex, Ez, Hy, m0 = memory_dEx_dz, m1 = memory_dEz_dx,
// m2 = memory_dHy_dx, m3 = memory_dHy_dz), seven arrays of N cells.  One
// forward step (electromag2.cu, FP32 build) is
//   H:  Hy' = [ring ? 0 : Hy] + dbHy (DEz - DEx)          i <= nx-2, k <= nz-2
//       DEx = rEx/kappa + m0',  m0' = b m0 + a rEx,  rEx = (Ex[k+1] - Ex) / dz
//       DEz = rEz/kappa_h + m1', m1' = bh m1 + ah rEz, rEz = (Ez[i+1] - Ez) / dx
//   E:  Ex' = Ex + dt (-aEx DHz + bEx DHx - dEx Ex - eEx Ez)   i >= 1, k >= 1
//       Ez' = Ez + dt (-aEz DHz + bEz DHx - dEz Ex - eEz Ez)
//       DHz = rHz/kappa + m3',  DHx = rHx/kappa_h + m2'  (backward differences of Hy')
//   source Ez' += f_n dt / eps33, then the Dirichlet ring on Ex', Ez'
// (0-based indices; Hy' on the ring rows i = 0, k = 0 is used by this step's
// E update and read as zero by the next H update).  The adjoint applies the
// transposes in reverse order, starting with the receiver residuals of the
// step.  The scatter of a stencil transpose becomes a
// gather over a scratch array: E^T leaves (lambda of rHz, rHx) x 1/dz, 1/dx
// per cell for H^T to gather, H^T leaves (lambda of rEx, rEz) x 1/dz, 1/dx
// for the gather into Ex, Ez -- which the next adjoint step's E^T performs
// before anything else reads those cells, so a step costs two grid passes.
// Gradients (FP32 sums within a checkpoint segment) are taken with respect
// to the eight per-cell coefficients aEx ... eEz; the host chains them to
// eps11, eps13, eps33, sig11, sig13, sig33.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ bool in_box(const BoxH& b, int i, int k) {
    return i >= b.i0 && i < b.i1 && k >= b.k0 && k < b.k1;
}

// gathered lambda of rEx / rEz (from H^T of the step after this one) at cell c
__device__ __forceinline__ float gather_x(const float* q0, size_t c, int k, int nx) {
    return (k >= 1 ? q0[c - nx] : 0.0f) - q0[c];
}
__device__ __forceinline__ float gather_z(const float* q1, size_t c, int i) {
    return (i >= 1 ? q1[c - 1] : 0.0f) - q1[c];
}

// ------------------------------------------------------------------ E^T
__global__ void __launch_bounds__(BX* BY) em_adj_e(EmAdjArgs A) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const E2Args<float>& a = A.a;
    const int nx = a.nx, nz = a.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = A.N;
    float* lam = A.lam;
    const float *q0 = A.scr + 2 * N, *q1 = A.scr + 3 * N;
    float lex = lam[c] + gather_x(q0, c, k, nx);
    float lez = lam[N + c] + gather_z(q1, c, i);
    if (A.dres) {  // receiver residuals of this step
        const float* res = A.dres + (size_t)(*A.base + A.j - 1) * 2 * A.nrec;
        for (int r = A.rfirst[c]; r >= 0; r = A.rnext[r]) {
            lex += res[r];
            lez += res[A.nrec + r];
        }
    }
    const bool ring = i == 0 || i == nx - 1 || k == 0 || k == nz - 1;
    if (ring) { lex = 0.f; lez = 0.f; }
    // every load precedes the first store (a store would hold later loads
    // behind it: the compiler cannot rule out aliasing between the slices)
    const bool src = i == a.isrc && k == a.jsrc && A.srcz;
    const double fsrc = src ? (double)(float)A.srcz[*A.base + A.j - 1] : 0.0;
    const double lez_src = (double)lez;
    float sz = 0.f, sx = 0.f;
    const bool upd = i >= 1 && k >= 1;
    const bool pml = !in_box(a.box, i, k);
    float g[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float m3 = 0.f, m2 = 0.f;
    if (upd) {
        const float dt = a.dt;
        const float* xp = A.xp;
        const float* xc = A.xc;
        const float exo = xp[c], ezo = xp[N + c];
        const float* hy = xc + 2 * N;
        float DHz = (hy[c] - hy[c - nx]) * a.dz;
        float DHx = (hy[c] - hy[c - 1]) * a.dx;
        if (pml) {
            DHz = DHz * a.cpml[0][c] + xc[6 * N + c];
            DHx = DHx * a.cpml[1][c] + xc[5 * N + c];
        }
        const float aEx = a.c[0][c], bEx = a.c[1][c], dEx = a.c[2][c], eEx = a.c[3][c];
        const float aEz = a.c[4][c], bEz = a.c[5][c], dEz = a.c[6][c], eEz = a.c[7][c];
        const float* G = A.grad;
        g[0] = G[c] - lex * dt * DHz;
        g[1] = G[N + c] + lex * dt * DHx;
        g[2] = G[2 * N + c] - lex * dt * exo;
        g[3] = G[3 * N + c] - lex * dt * ezo;
        g[4] = G[4 * N + c] - lez * dt * DHz;
        g[5] = G[5 * N + c] + lez * dt * DHx;
        g[6] = G[6 * N + c] - lez * dt * exo;
        g[7] = G[7 * N + c] - lez * dt * ezo;
        const float lDHz = -dt * (aEx * lex + aEz * lez);
        const float lDHx = dt * (bEx * lex + bEz * lez);
        float lrz = lDHz, lrx = lDHx;
        if (pml) {
            const float M3 = lam[6 * N + c] + lDHz, M2 = lam[5 * N + c] + lDHx;
            lrz = a.cpml[0][c] * lDHz + a.cpml[2][c] * M3;
            lrx = a.cpml[1][c] * lDHx + a.cpml[3][c] * M2;
            m3 = a.cpml[4][c] * M3;
            m2 = a.cpml[5][c] * M2;
        }
        sz = lrz * a.dz;
        sx = lrx * a.dx;
        const float nlex = lex - dt * (dEx * lex + dEz * lez);
        const float nlez = lez - dt * (eEx * lex + eEz * lez);
        lex = nlex;
        lez = nlez;
    }
    // ---- stores
    if (src) *A.gsrc += lez_src * fsrc;
    if (upd) {
#pragma unroll
        for (int q = 0; q < 8; ++q) A.grad[q * N + c] = g[q];
        if (pml) {
            lam[6 * N + c] = m3;
            lam[5 * N + c] = m2;
        }
    }
    lam[c] = lex;
    lam[N + c] = lez;
    A.scr[c] = sz;
    A.scr[N + c] = sx;
}

// ------------------------------------------------- gather into Hy, then H^T
__global__ void __launch_bounds__(BX* BY) em_adj_h(EmAdjArgs A) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const E2Args<float>& a = A.a;
    const int nx = a.nx, nz = a.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = A.N;
    const float *sz = A.scr, *sx = A.scr + N;
    float* lam = A.lam;
    const float lhy = lam[2 * N + c] + sz[c] - (k + 1 < nz ? sz[c + nx] : 0.0f) + sx[c] -
                      (i + 1 < nx ? sx[c + 1] : 0.0f);
    float q0 = 0.f, q1 = 0.f, nl = 0.f;
    if (i <= nx - 2 && k <= nz - 2) {
        const float lD = a.dbHy * lhy;
        float lrz = -lD, lrx = lD;  // lambda of rEx (via -DEx) and of rEz (via +DEz)
        if (!in_box(a.box, i, k)) {
            float* l0 = lam + 3 * N + c;
            float* l1 = lam + 4 * N + c;
            const float M0 = *l0 - lD, M1 = *l1 + lD;
            lrz = a.cpml[0][c] * (-lD) + a.cpml[2][c] * M0;
            lrx = a.cpml[1][c] * lD + a.cpml[3][c] * M1;
            const float n0 = a.cpml[4][c] * M0, n1 = a.cpml[5][c] * M1;  // both loads before the stores
            *l0 = n0;
            *l1 = n1;
        }
        q0 = lrz * a.dz;
        q1 = lrx * a.dx;
        nl = (i == 0 || k == 0) ? 0.f : lhy;
    }
    lam[2 * N + c] = nl;
    A.scr[2 * N + c] = q0;
    A.scr[3 * N + c] = q1;
}

// pending gather of H^T into Ex, Ez (host test hook only; the sweep leaves
// it to the next step's E^T)
__global__ void __launch_bounds__(BX* BY) em_adj_flush(EmAdjArgs A) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const int nx = A.a.nx, nz = A.a.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = A.N;
    A.lam[c] += gather_x(A.scr + 2 * N, c, k, nx);
    A.lam[N + c] += gather_z(A.scr + 3 * N, c, i);
}

// ------------------------------------------- out-of-place recompute step
// The arithmetic of electromag2.cu's FP32 kernels, reading x_{j-1} from
// `in` and writing x_j to `out`.  Memories are written only on cells outside
// the inert box (inside it they stay zero from the buffer's allocation).
__global__ void __launch_bounds__(BX* BY) em_oop_h(EmOopArgs O) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const E2Args<float>& a = O.a;
    const int nx = a.nx, nz = a.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = O.N;
    const float *in = O.in;
    float* out = O.out;
    const bool pml = !in_box(a.box, i, k);
    if (i == nx - 1 || k == nz - 1) {
        out[2 * N + c] = 0.f;
        if (pml) { out[3 * N + c] = in[3 * N + c]; out[4 * N + c] = in[4 * N + c]; }
        return;
    }
    const float *Ex = in, *Ez = in + N;
    float dEx_dz = (Ex[c + nx] - Ex[c]) * a.dz;
    float dEz_dx = (Ez[c + 1] - Ez[c]) * a.dx;
    float M0 = 0.f, M1 = 0.f;
    if (pml) {
        M0 = a.cpml[4][c] * in[3 * N + c] + a.cpml[2][c] * dEx_dz;
        M1 = a.cpml[5][c] * in[4 * N + c] + a.cpml[3][c] * dEz_dx;
        dEz_dx = dEz_dx * a.cpml[1][c] + M1;
        dEx_dz = dEx_dz * a.cpml[0][c] + M0;
    }
    const float hy = (i == 0 || k == 0) ? 0.f : in[2 * N + c];
    // stores after every load
    if (pml) {
        out[3 * N + c] = M0;
        out[4 * N + c] = M1;
    }
    out[2 * N + c] = hy + a.dbHy * (dEz_dx - dEx_dz);
}

__global__ void __launch_bounds__(BX* BY) em_oop_e(EmOopArgs O) {
    const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
    const E2Args<float>& a = O.a;
    const int nx = a.nx, nz = a.nz;
    if (i >= nx || k >= nz) return;
    const size_t c = (size_t)i + (size_t)nx * k, N = O.N;
    const float* in = O.in;
    float* out = O.out;
    const bool pml = !in_box(a.box, i, k);
    float ex = in[c], ez = in[N + c];
    float M2 = 0.f, M3 = 0.f;  // stored after every load
    if (i >= 1 && k >= 1) {
        const float* Hy = out + 2 * N;
        float dHy_dz = (Hy[c] - Hy[c - nx]) * a.dz;
        float dHy_dx = (Hy[c] - Hy[c - 1]) * a.dx;
        if (pml) {
            M2 = a.cpml[5][c] * in[5 * N + c] + a.cpml[3][c] * dHy_dx;
            M3 = a.cpml[4][c] * in[6 * N + c] + a.cpml[2][c] * dHy_dz;
            dHy_dz = dHy_dz * a.cpml[0][c] + M3;
            dHy_dx = dHy_dx * a.cpml[1][c] + M2;
        }
        const float aEx = a.c[0][c], bEx = a.c[1][c], dEx = a.c[2][c], eEx = a.c[3][c];
        const float aEz = a.c[4][c], bEz = a.c[5][c], dEz = a.c[6][c], eEz = a.c[7][c];
        const float exo = ex, ezo = ez;
        ez = ezo + (-(aEz * dHy_dz) + bEz * dHy_dx - dEz * exo - eEz * ezo) * a.dt;
        ex = exo + (-(aEx * dHy_dz) + bEx * dHy_dx - dEx * exo - eEx * ezo) * a.dt;
    } else if (pml) {
        M2 = in[5 * N + c];
        M3 = in[6 * N + c];
    }
    if (i == a.isrc && k == a.jsrc && O.srcz) ez = ez + (float)O.srcz[*O.base + O.j - 1] * a.dt / a.c[9][c];
    if (i == 0 || i == nx - 1 || k == 0 || k == nz - 1) { ex = 0.f; ez = 0.f; }
    if (pml) {
        out[5 * N + c] = M2;
        out[6 * N + c] = M3;
    }
    out[c] = ex;
    out[N + c] = ez;
}

}  // namespace

void em2_adjoint_step(const EmAdjArgs& A, cudaStream_t st) {
    const dim3 blk(BX, BY), grd((A.a.nx + BX - 1) / BX, (A.a.nz + BY - 1) / BY);
    em_adj_e<<<grd, blk, 0, st>>>(A);
    em_adj_h<<<grd, blk, 0, st>>>(A);
}

void em2_adjoint_flush(const EmAdjArgs& A, cudaStream_t st) {
    const dim3 blk(BX, BY), grd((A.a.nx + BX - 1) / BX, (A.a.nz + BY - 1) / BY);
    em_adj_flush<<<grd, blk, 0, st>>>(A);
}

void em2_recompute_step(const EmOopArgs& O, cudaStream_t st) {
    const dim3 blk(BX, BY), grd((O.a.nx + BX - 1) / BX, (O.a.nz + BY - 1) / BY);
    em_oop_h<<<grd, blk, 0, st>>>(O);
    em_oop_e<<<grd, blk, 0, st>>>(O);
}
