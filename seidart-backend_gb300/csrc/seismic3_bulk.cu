// seismic3_bulk.cu -- FP32 3D elastic stress half-step with the per-cell
// coefficients staged in shared memory by one bulk copy per CTA.
//
// Same arithmetic as the FP32 stress loops of seismic3.cu
// (src/fortran/cpmlfdtd.f08:1761-1992).  What changes is where the 27
// read-only per-cell coefficients (21 C_ij and 6 attenuation factors
// 1/(1 + gamma dt)) live:
//   * at set-up they are repacked tile-major: for every 32 x 8 tile of one
//     z plane a contiguous block [27][8][32] floats (27,648 bytes);
//   * a CTA owns one tile: its first thread starts a single cp.async.bulk of
//     that block into shared memory, then every thread issues its velocity
//     stencil loads and old stresses and forms its derivatives while the
//     copy is in flight, waits on the mbarrier (bounded) and finishes the
//     update reading C_ij from shared memory.
// The bytes in flight for the coefficient stream cost no registers, which is
// what the register-bound one-cell kernels lack: they stall on load latency
// with HBM a third busy.  A wait that gives up sets the solver's error word
// and skips the update; the CTA still lets its copy land before exiting.
#include <algorithm>

#include "s3_velocity.cuh"

namespace {

using namespace s3;

constexpr int BX = 32, BY = 8, NT = BX * BY, NCOEF = 27;
constexpr unsigned TILE_BYTES = NCOEF * NT * sizeof(float);

// stress store: streaming (evict-first) when the next reader is the next
// launch, plain when other CTAs of the same launch read it back from L2
template <bool STREAM>
__device__ __forceinline__ void st_sig(float* p, float v) {
    if constexpr (STREAM) __stcs(p, v);
    else *p = v;
}

// The bounded wait of a staged CTA.  On give-up the CTA sets the solver's
// error word and its first thread waits again, with the far larger bound
// WAIT_LAND, for the copies it issued to land, so that no copy writes into
// shared memory after the CTA has retired (the copies read this GPU's own
// HBM, so they finish within microseconds whenever the GPU makes progress).
// `probe` > 0 (a test hook, one CTA): the barrier was armed with that many
// bytes more than the copies bring, so the first wait runs out; the give-up
// path then completes the missing bytes itself before it drains.
constexpr int WAIT_LAND = 1 << 26;
__device__ __forceinline__ bool staged_wait(const S3Args<float>& A, unsigned long long* bar, int tid, int probe,
                                            unsigned parity = 0) {
    if (mbar_wait_bounded(bar, parity, A.wait_limit)) return true;
    if (tid == 0) {
        if (A.err) atomicExch(A.err, 1);
        if (probe > 0) mbar_complete_tx(bar, (unsigned)probe);
        mbar_wait_bounded(bar, parity, WAIT_LAND);
    }
    return false;
}


__global__ void __launch_bounds__(NT) s3b_pack(S3Args<float> A, float* P) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    const size_t t = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * k);
    float* dst = P + t * (NCOEF * NT) + threadIdx.y * BX + threadIdx.x;
    const bool in = i < A.nx && j < A.ny;
    const size_t c = in ? (size_t)i + (size_t)A.nx * ((size_t)j + (size_t)A.ny * k) : 0;
#pragma unroll
    for (int q = 0; q < 21; ++q) dst[q * NT] = in ? A.C[q][c] : 0.0f;
#pragma unroll
    for (int q = 0; q < 6; ++q) dst[(21 + q) * NT] = in ? A.g[q][c] : 0.0f;
}

// L2 prefetch of everything the CTA `dist` tiles later in launch order will
// read: its coefficient block, old stresses and velocities, and on shell
// tiles the CPML memories and coefficients.  A hint only: no registers or
// shared memory stay allocated for it.
__device__ __forceinline__ void s3b_prefetch(const S3Args<float>& A, int dist, int tid) {
    (void)dist;  // A.pf_d holds it split into tile offsets
    int tx, ty, k;
    if (!tile_ahead(A.pf_d, tx, ty, k)) return;
    if (k < 1 || k > A.nz - 2) return;
    const size_t lin = (size_t)tx + (size_t)gridDim.x * ((size_t)ty + (size_t)gridDim.y * k);
    if (A.mat_ids) {
        if (tid < NT / 128) pf_l2(A.mat_ids + lin * NT + tid * 128);  // the tile's material bytes
    } else if (tid < NCOEF * NT / 32) {
        pf_l2(A.packed + lin * (NCOEF * NT) + tid * 32);
    }
    pf_tile_rows(A.f, 9, tx, ty, k, A.nx, A.ny, tid, NT);
    if (!tile_in_box(A.box, tx, ty, k, A.nx, A.ny)) {
        if (A.mem_merged) {
            // the 21 memories the merged layout advances: slots 0..17, 20, 23, 26
            pf_tile_rows(A.mem, 18, tx, ty, k, A.nx, A.ny, tid, NT);
            for (int f = 0; f < 3; ++f) pf_tile_rows(A.mem + 20 + 3 * f, 1, tx, ty, k, A.nx, A.ny, tid, NT);
        } else {
            pf_tile_rows(A.mem, 36, tx, ty, k, A.nx, A.ny, tid, NT);
        }
        pf_cpml_tile(A, tx, ty, k, tid, NT);
    }
}

// Everything after the bulk copy is started: stencil loads and derivatives
// (overlapping the copy), the bounded wait, then the update with C_ij from
// shared memory.  LEAN drops the clamps, loop-bound tests and CPML branches.
template <bool LEAN>
__device__ __forceinline__ void stress_tile(const S3Args<float>& A, const float* coef, unsigned long long* bar, int tid,
                                            int k) {
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    const int gx = blockIdx.x * BX + threadIdx.x, gy = blockIdx.y * BY + threadIdx.y;
    bool L1 = true, L2 = true, L3 = true, L4 = true, active = true;
    if (!LEAN) {
        const bool x14 = gx >= 1 && gx <= nx - 3, x23 = gx >= 2 && gx <= nx - 2;
        const bool y13 = gy >= 2 && gy <= ny - 2, y24 = gy >= 1 && gy <= ny - 3;
        const bool z12 = k >= 2 && k <= nz - 2, z34 = k >= 1 && k <= nz - 3;
        L1 = x14 && y13 && z12; L2 = x23 && y24 && z12; L3 = x23 && y13 && z34; L4 = x14 && y24 && z34;
        active = gx < nx && gy < ny && (L1 || L2 || L3 || L4);
    }
    const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
    const size_t c = active ? (size_t)gx + sy * gy + sz * k : 0;
    float so[6], fx[3], bx[3], fy[3], by[3], fz[3], bz[3];
    if (active) {
        long ox[4] = {-2, -1, 1, 2}, oy[4] = {-2 * (long)sy, -(long)sy, (long)sy, 2 * (long)sy},
             oz[4] = {-2 * (long)sz, -(long)sz, (long)sz, 2 * (long)sz};
        if (!LEAN) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int d = q < 2 ? q - 2 : q - 1;
                ox[q] = (long)cl(gx + d, 0, nx - 1) - gx;
                oy[q] = ((long)cl(gy + d, 0, ny - 1) - gy) * (long)sy;
                oz[q] = ((long)cl(k + d, 0, nz - 1) - k) * (long)sz;
            }
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) so[q] = __ldcs(A.f[3 + q] + c);
        const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float* p = A.f[f] + c;
            const float a0 = __ldg(p);
            const float xm2 = __ldg(p + ox[0]), xm1 = __ldg(p + ox[1]), xp1 = __ldg(p + ox[2]), xp2 = __ldg(p + ox[3]);
            const float ym2 = __ldg(p + oy[0]), ym1 = __ldg(p + oy[1]), yp1 = __ldg(p + oy[2]), yp2 = __ldg(p + oy[3]);
            const float zm2 = __ldg(p + oz[0]), zm1 = __ldg(p + oz[1]), zp1 = __ldg(p + oz[2]), zp2 = __ldg(p + oz[3]);
            fx[f] = (27.0f * (xp1 - a0) - (xp2 - xm1)) * hx;
            bx[f] = (27.0f * (a0 - xm1) - (xp1 - xm2)) * hx;
            fy[f] = (27.0f * (yp1 - a0) - (yp2 - ym1)) * hy;
            by[f] = (27.0f * (a0 - ym1) - (yp1 - ym2)) * hy;
            fz[f] = (27.0f * (zp1 - a0) - (zp2 - zm1)) * hz;
            bz[f] = (27.0f * (a0 - zm1) - (zp1 - zm2)) * hz;
        }
    }
    if (!staged_wait(A, bar, tid, 0)) return;
    if (!active) return;
    const auto CR = [&](int q) { return coef[q * NT + tid]; };
    const auto GM = [&](int q) { return coef[(21 + q) * NT + tid]; };
    const bool pml = !LEAN && !(A.box.i0 <= gx && gx < A.box.i1 && A.box.j0 <= gy && gy < A.box.j1 &&
                                A.box.k0 <= k && k < A.box.k1);
    const float dt = A.dt;
    // C index: 0 c11 1 c12 2 c13 3 c14 4 c15 5 c16 6 c22 7 c23 8 c24 9 c25 10 c26
    //          11 c33 12 c34 13 c35 14 c36 15 c44 16 c45 17 c46 18 c55 19 c56 20 c66
    // so order: sigma xx xy xz yy yz zz ; gamma order: x y z xy yz xz
    if (L1) {
        float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {bz[0], bz[1], bz[2]};
        if (pml) loop_cpml<1>(A, c, ex, ey, ez);
        __stcs(A.f[3] + c, stress_new(CR, so[0], GM(0), 0, 1, 2, 3, 4, 5, dt, ex, ey, ez));
        __stcs(A.f[6] + c, stress_new(CR, so[3], GM(1), 1, 6, 7, 8, 9, 10, dt, ex, ey, ez));
        __stcs(A.f[8] + c, stress_new(CR, so[5], GM(2), 2, 7, 11, 12, 13, 14, dt, ex, ey, ez));
    }
    if (L2) {
        float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {bz[0], bz[1], bz[2]};
        if (pml) loop_cpml<2>(A, c, ex, ey, ez);
        __stcs(A.f[4] + c, stress_new(CR, so[1], GM(3), 5, 10, 14, 17, 19, 20, dt, ex, ey, ez));
    }
    if (L3) {
        float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {fz[0], fz[1], fz[2]};
        if (pml) loop_cpml<3>(A, c, ex, ey, ez);
        __stcs(A.f[5] + c, stress_new(CR, so[2], GM(5), 4, 9, 13, 16, 18, 19, dt, ex, ey, ez));
    }
    if (L4) {
        float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {fz[0], fz[1], fz[2]};
        if (pml) loop_cpml<4>(A, c, ex, ey, ez);
        __stcs(A.f[7] + c, stress_new(CR, so[4], GM(4), 3, 8, 12, 15, 16, 17, dt, ex, ey, ez));
    }
}

template <int MINB>
__global__ void __launch_bounds__(NT, MINB) s3b_stress(S3Args<float> A) {
    extern __shared__ __align__(128) float coef[];  // [27][NT]
    __shared__ __align__(8) unsigned long long bar;
    const int k = blockIdx.z, nx = A.nx, ny = A.ny, nz = A.nz;
    const int tid = threadIdx.y * BX + threadIdx.x;
    if (A.prefetch > 0) s3b_prefetch(A, A.prefetch, tid);
    if (k < 1 || k > nz - 2) return;  // planes 0 and nz-1 hold no stress update
    if (tid == 0) {
        const size_t t = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * k);
        mbar_init(&bar, 1);
        mbar_expect_tx(&bar, TILE_BYTES);
        bulk_g2s(coef, A.packed + t * (NCOEF * NT), TILE_BYTES, &bar);
    }
    __syncthreads();
    // lean tiles: wholly inside the inert interior box and two cells from
    // every face, so all four loops apply, no index is clamped and no CPML
    // branch is taken
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const bool lean = x0 >= 2 && x0 + BX - 1 <= nx - 3 && y0 >= 2 && y0 + BY - 1 <= ny - 3 && k >= 2 && k <= nz - 3 &&
                      x0 >= A.box.i0 && x0 + BX <= A.box.i1 && y0 >= A.box.j0 && y0 + BY <= A.box.j1 &&
                      k >= A.box.k0 && k < A.box.k1;
    if (lean) stress_tile<true>(A, coef, &bar, tid, k);
    else stress_tile<false>(A, coef, &bar, tid, k);
}

// ------------------------------------------------ fully staged variant
// Everything the update reads per cell arrives by asynchronous copies into
// shared memory before any thread computes: the coefficient block (one bulk
// copy), the six old stresses (32 x 8 tensor tiles), the three velocities of
// plane k with a 4-cell x / 2-cell y halo (40 x 12 tiles, from x0-4 so every
// box starts 16-byte aligned) and of planes k-2, k-1, k+1, k+2 (32 x 8
// tiles).  22 copies, issued one per lane of warp 0, one mbarrier.  Boxes
// reaching outside the grid read zeros there; those values only enter
// derivatives that the cell's loops do not use (as the clamped loads of the
// register kernels).  Only CPML memories and coefficients on shell tiles
// still travel through registers.
constexpr int VHW = BX + 8, VHH = BY + 4;       // halo box 40 x 12
constexpr int XS_SIG = NCOEF * NT;              // [6][NT]
constexpr int XS_VH = XS_SIG + 6 * NT;          // [3][VHH][VHW]
constexpr int XS_VZ = XS_VH + 3 * VHW * VHH;    // [3][4][NT]: z = k-2, k-1, k+1, k+2
constexpr int XS_TOTAL = XS_VZ + 12 * NT;
constexpr unsigned XS_BYTES = XS_TOTAL * sizeof(float);  // 51,840
// Material-indexed model: the coefficient block is replaced by the material
// table ([S3_MAXMAT][27] floats) and the tile's material bytes ([NT]); the
// stresses and velocities follow at a 128-byte aligned offset.
constexpr int XI_TAB = 0;
constexpr int XI_ID = S3_MAXMAT * NCOEF;                 // 864 floats
constexpr int XI_SIG = XI_ID + NT / 4;                   // 928 floats (3,712 bytes)
constexpr int XI_TOTAL = XI_SIG + (XS_TOTAL - XS_SIG);
constexpr unsigned XI_BYTES = XI_TOTAL * sizeof(float);  // 27,904
constexpr unsigned XS_FIELD_BYTES = XS_BYTES - TILE_BYTES;  // stresses and velocities of a tile
static_assert((XI_SIG * sizeof(float)) % 128 == 0, "tensor-copy destinations need 128-byte alignment");

// IDX: the material-indexed layout (coefficients from the material table)
template <bool LEAN, bool STREAM = true, bool IDX = false, bool MERGED = false>
__device__ __forceinline__ void staged_tile(const S3Args<float>& A, const float* sm, unsigned long long* bar, int tid,
                                            int x0, int y0, int k, int probe, unsigned parity = 0) {
    constexpr int SIG = IDX ? XI_SIG : XS_SIG, VH = SIG + 6 * NT, VZ = VH + 3 * VHW * VHH;
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
    bool L1 = true, L2 = true, L3 = true, L4 = true, active = true;
    if (!LEAN) {
        const bool x14 = gx >= 1 && gx <= nx - 3, x23 = gx >= 2 && gx <= nx - 2;
        const bool y13 = gy >= 2 && gy <= ny - 2, y24 = gy >= 1 && gy <= ny - 3;
        const bool z12 = k >= 2 && k <= nz - 2, z34 = k >= 1 && k <= nz - 3;
        L1 = x14 && y13 && z12; L2 = x23 && y24 && z12; L3 = x23 && y13 && z34; L4 = x14 && y24 && z34;
        active = gx < nx && gy < ny && (L1 || L2 || L3 || L4);
    }
    if (!staged_wait(A, bar, tid, probe, parity)) return;
    if (!active) return;
    const size_t c = (size_t)gx + (size_t)nx * ((size_t)gy + (size_t)ny * k);
    const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
    float fx[3], bx[3], fy[3], by[3], fz[3], bz[3];
    const int hc = (threadIdx.y + 2) * VHW + threadIdx.x + 4;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        const float* H = sm + VH + f * VHW * VHH + hc;
        const float* Z = sm + VZ + f * 4 * NT + tid;
        const float a0 = H[0];
        const float xm2 = H[-2], xm1 = H[-1], xp1 = H[1], xp2 = H[2];
        const float ym2 = H[-2 * VHW], ym1 = H[-VHW], yp1 = H[VHW], yp2 = H[2 * VHW];
        const float zm2 = Z[0], zm1 = Z[NT], zp1 = Z[2 * NT], zp2 = Z[3 * NT];
        fx[f] = (27.0f * (xp1 - a0) - (xp2 - xm1)) * hx;
        bx[f] = (27.0f * (a0 - xm1) - (xp1 - xm2)) * hx;
        fy[f] = (27.0f * (yp1 - a0) - (yp2 - ym1)) * hy;
        by[f] = (27.0f * (a0 - ym1) - (yp1 - ym2)) * hy;
        fz[f] = (27.0f * (zp1 - a0) - (zp2 - zm1)) * hz;
        bz[f] = (27.0f * (a0 - zm1) - (zp1 - zm2)) * hz;
    }
    const float* so = sm + SIG + tid;  // old stress q at so[q * NT]
    // coefficient q of this cell: its slot of the tile block, or of its
    // material's row of the table (the same FP32 values)
    const float* cf = IDX ? sm + XI_TAB + NCOEF * reinterpret_cast<const unsigned char*>(sm + XI_ID)[tid] : sm + tid;
    constexpr int CS = IDX ? 1 : NT;
    const auto CR = [&](int q) { return cf[q * CS]; };
    const auto GM = [&](int q) { return cf[(21 + q) * CS]; };
    const bool pml = !LEAN && !(A.box.i0 <= gx && gx < A.box.i1 && A.box.j0 <= gy && gy < A.box.j1 &&
                                A.box.k0 <= k && k < A.box.k1);
    const float dt = A.dt;
    // C index: 0 c11 1 c12 2 c13 3 c14 4 c15 5 c16 6 c22 7 c23 8 c24 9 c25 10 c26
    //          11 c33 12 c34 13 c35 14 c36 15 c44 16 c45 17 c46 18 c55 19 c56 20 c66
    // old stress order: xx xy xz yy yz zz ; gamma order: x y z xy yz xz
    // shell cells: the memories of loops 1 and 2 are loaded together, and
    // those of loops 3 and 4 together after the first pair's stores, so a
    // cell waits for two DRAM round trips instead of four.
    // MERGED: the derivatives two loops share -- the same stencil with the
    // same C-PML coefficients -- advance one memory instead of two: forward x
    // with the half-grid coefficients (loops 1 and 4), backward x full (2 and
    // 3), backward y full (1 and 3), forward y half (2 and 4), forward z half
    // (3 and 4).  Where both loops of a pair update a cell their two memories
    // start at zero and advance with the same values, so they stay equal; the
    // first loop of the pair that applies at the cell advances the shared
    // memory and the other reads the advanced value.  Loop 1's nine slots,
    // loop 2's nine and loop 3's three z slots hold the 21 memories, all
    // loaded at once (one round trip); seidart_solver_get_memory rebuilds the
    // reference's 36 arrays from them.
    CpmlPair P{};
    float ma[9], mb[9], mz[3];
    if (pml) {
        P = cpml_pair_at(A, c, gx, gy, k);
        if (MERGED) {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                ma[q] = A.mem[q][c];
                mb[q] = A.mem[9 + q][c];
            }
#pragma unroll
            for (int f = 0; f < 3; ++f) mz[f] = A.mem[18 + 3 * f + 2][c];
        } else {
            if (L1) cpml_load<1>(A, c, ma);
            if (L2) cpml_load<2>(A, c, mb);
        }
    }
    if (L1) {
        float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {bz[0], bz[1], bz[2]};
        if (pml) {
            cpml_update<1>(P, ma, ex, ey, ez);
            if (!MERGED) cpml_store<1>(A, c, ma);
        }
        st_sig<STREAM>(A.f[3] + c, stress_new(CR, so[0], GM(0), 0, 1, 2, 3, 4, 5, dt, ex, ey, ez));
        st_sig<STREAM>(A.f[6] + c, stress_new(CR, so[3 * NT], GM(1), 1, 6, 7, 8, 9, 10, dt, ex, ey, ez));
        st_sig<STREAM>(A.f[8] + c, stress_new(CR, so[5 * NT], GM(2), 2, 7, 11, 12, 13, 14, dt, ex, ey, ez));
    }
    if (L2) {
        float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {bz[0], bz[1], bz[2]};
        if (pml) {
            cpml_update<2>(P, mb, ex, ey, ez);
            if (!MERGED) cpml_store<2>(A, c, mb);
        }
        st_sig<STREAM>(A.f[4] + c, stress_new(CR, so[NT], GM(3), 5, 10, 14, 17, 19, 20, dt, ex, ey, ez));
    }
    if (MERGED) {
        // advance memory m with coefficient triple p unless the pair's other
        // loop already did (done), then rescale the derivative
        const auto adv = [](float& m, const CpmlC& p, float& g, bool done) {
            if (!done) m = p.b * m + p.a * g;
            g = g * p.k + m;
        };
        if (L3) {
            float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {fz[0], fz[1], fz[2]};
            if (pml) {
#pragma unroll
                for (int f = 0; f < 3; ++f) {
                    adv(mb[3 * f], P.f, ex[f], L2);      // backward x, full: loop 2's memory
                    adv(ma[3 * f + 1], P.f, ey[f], L1);  // backward y, full: loop 1's memory
                    adv(mz[f], P.h, ez[f], false);       // forward z, half: loop 3's own
                }
            }
            st_sig<STREAM>(A.f[5] + c, stress_new(CR, so[2 * NT], GM(5), 4, 9, 13, 16, 18, 19, dt, ex, ey, ez));
        }
        if (L4) {
            float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {fz[0], fz[1], fz[2]};
            if (pml) {
#pragma unroll
                for (int f = 0; f < 3; ++f) {
                    adv(ma[3 * f], P.h, ex[f], L1);      // forward x, half: loop 1's memory
                    adv(mb[3 * f + 1], P.h, ey[f], L2);  // forward y, half: loop 2's memory
                    adv(mz[f], P.h, ez[f], L3);          // forward z, half: loop 3's memory
                }
            }
            st_sig<STREAM>(A.f[7] + c, stress_new(CR, so[4 * NT], GM(4), 3, 8, 12, 15, 16, 17, dt, ex, ey, ez));
        }
        if (pml) {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                A.mem[q][c] = ma[q];
                A.mem[9 + q][c] = mb[q];
            }
#pragma unroll
            for (int f = 0; f < 3; ++f) A.mem[18 + 3 * f + 2][c] = mz[f];
        }
        return;
    }
    if (pml) {
        if (L3) cpml_load<3>(A, c, ma);
        if (L4) cpml_load<4>(A, c, mb);
    }
    if (L3) {
        float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {fz[0], fz[1], fz[2]};
        if (pml) {
            cpml_update<3>(P, ma, ex, ey, ez);
            cpml_store<3>(A, c, ma);
        }
        st_sig<STREAM>(A.f[5] + c, stress_new(CR, so[2 * NT], GM(5), 4, 9, 13, 16, 18, 19, dt, ex, ey, ez));
    }
    if (L4) {
        float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {fz[0], fz[1], fz[2]};
        if (pml) {
            cpml_update<4>(P, mb, ex, ey, ez);
            cpml_store<4>(A, c, mb);
        }
        st_sig<STREAM>(A.f[7] + c, stress_new(CR, so[4 * NT], GM(4), 3, 8, 12, 15, 16, 17, dt, ex, ey, ez));
    }
}

// Arm the CTA's barrier and issue the 22 copies of one staged stress tile
// (tile tx, ty of plane k; `lin` its index in the packed coefficient array),
// one per lane of warp 0.  `probe` extra bytes are armed on top (test hook).
// the 22 copies alone (lanes 0..21 of warp 0), on a barrier already armed
__device__ __forceinline__ void stress_copies_issue(const S3Args<float>& A, const S3XMaps& M, float* sm,
                                                    unsigned long long* bar, int tid, int x0, int y0, int k,
                                                    size_t lin) {
    if (tid < 22) {
        if (tid == 0) {
            bulk_g2s(sm, A.packed + lin * (NCOEF * NT), TILE_BYTES, bar);
        } else if (tid <= 6) {
            tma_load3(sm + XS_SIG + (tid - 1) * NT, &M.sig[tid - 1], x0, y0, k, bar);
        } else if (tid <= 9) {
            tma_load3(sm + XS_VH + (tid - 7) * VHW * VHH, &M.vh[tid - 7], x0 - 4, y0 - 2, k, bar);
        } else {
            const int q = tid - 10, f = q >> 2, zi = q & 3;
            const int dz = zi < 2 ? zi - 2 : zi - 1;
            tma_load3(sm + XS_VZ + q * NT, &M.vp[f], x0, y0, k + dz, bar);
        }
    }
}

template <bool IDX = false>
__device__ __forceinline__ void stress_copies(const S3Args<float>& A, const S3XMaps& M, float* sm,
                                              unsigned long long* bar, int tid, int x0, int y0, int k, size_t lin,
                                              int probe) {
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_expect_tx(bar, (IDX ? (unsigned)A.mat_tab_bytes + NT + XS_FIELD_BYTES : XS_BYTES) + (unsigned)probe);
    }
    __syncthreads();
    if (IDX) {
        // the material table (lane 0), the tile's material bytes (lane 22),
        // the stresses and velocities (lanes 1..21) as in the block layout
        if (tid == 0) {
            bulk_g2s(sm + XI_TAB, A.mat_tab, (unsigned)A.mat_tab_bytes, bar);
        } else if (tid == 22) {
            bulk_g2s(sm + XI_ID, A.mat_ids + lin * NT, NT, bar);
        } else if (tid <= 6) {
            tma_load3(sm + XI_SIG + (tid - 1) * NT, &M.sig[tid - 1], x0, y0, k, bar);
        } else if (tid <= 9) {
            tma_load3(sm + XI_SIG + 6 * NT + (tid - 7) * VHW * VHH, &M.vh[tid - 7], x0 - 4, y0 - 2, k, bar);
        } else if (tid < 22) {
            const int q = tid - 10, f = q >> 2, zi = q & 3;
            const int dz = zi < 2 ? zi - 2 : zi - 1;
            tma_load3(sm + XI_SIG + 6 * NT + 3 * VHW * VHH + q * NT, &M.vp[f], x0, y0, k + dz, bar);
        }
        return;
    }
    if (tid < 22) {
        if (A.l2_hint && tid <= 6) {
            // the coefficient block and the old stresses are read once
            const uint64_t pol = policy_evict_first();
            if (tid == 0) bulk_g2s_hint(sm, A.packed + lin * (NCOEF * NT), TILE_BYTES, bar, pol);
            else tma_load3_hint(sm + XS_SIG + (tid - 1) * NT, &M.sig[tid - 1], x0, y0, k, bar, pol);
        } else if (tid == 0) {
            bulk_g2s(sm, A.packed + lin * (NCOEF * NT), TILE_BYTES, bar);
        } else if (tid <= 6) {
            tma_load3(sm + XS_SIG + (tid - 1) * NT, &M.sig[tid - 1], x0, y0, k, bar);
        } else if (tid <= 9) {
            tma_load3(sm + XS_VH + (tid - 7) * VHW * VHH, &M.vh[tid - 7], x0 - 4, y0 - 2, k, bar);
        } else {
            const int q = tid - 10, f = q >> 2, zi = q & 3;
            const int dz = zi < 2 ? zi - 2 : zi - 1;
            tma_load3(sm + XS_VZ + q * NT, &M.vp[f], x0, y0, k + dz, bar);
        }
    }
}

__device__ __forceinline__ bool lean_stress_tile(const S3Args<float>& A, int x0, int y0, int k) {
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    return x0 >= 2 && x0 + BX - 1 <= nx - 3 && y0 >= 2 && y0 + BY - 1 <= ny - 3 && k >= 2 && k <= nz - 3 &&
           x0 >= A.box.i0 && x0 + BX <= A.box.i1 && y0 >= A.box.j0 && y0 + BY <= A.box.j1 && k >= A.box.k0 &&
           k < A.box.k1;
}

// the test hook arms extra bytes on one CTA: the first tile of plane 2
__device__ __forceinline__ int probe_bytes(const S3Args<float>& A, int tx, int ty, int k) {
    return (A.wait_probe > 0 && tx == 0 && ty == 0 && k == 2) ? A.wait_probe : 0;
}

template <int MINB, bool IDX = false, bool MERGED = false>
__global__ void __launch_bounds__(NT, MINB) s3x_stress(S3Args<float> A, const __grid_constant__ S3XMaps M) {
    extern __shared__ __align__(128) float sm[];
    __shared__ __align__(8) unsigned long long bar;
    const int k = blockIdx.z, nz = A.nz;
    const int tid = threadIdx.y * BX + threadIdx.x;
    if (A.prefetch > 0) s3b_prefetch(A, A.prefetch, tid);
    if (k < 1 || k > nz - 2) return;  // planes 0 and nz-1 hold no stress update
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int probe = probe_bytes(A, blockIdx.x, blockIdx.y, k);
    stress_copies<IDX>(A, M, sm, &bar, tid, x0, y0, k,
                       blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * k), probe);
    if (lean_stress_tile(A, x0, y0, k)) staged_tile<true, true, IDX, MERGED>(A, sm, &bar, tid, x0, y0, k, probe);
    else staged_tile<false, true, IDX, MERGED>(A, sm, &bar, tid, x0, y0, k, probe);
}

// ------------------------------------------------ fused step (wavefront)
// Both half-steps of one time step in one launch.  Work items are (plane p,
// tile) in plane-major order and are handed out by an atomic ticket, so an
// item is only ever started after every item before it has been started:
//   * stress half-step of the tile at plane p (the staged tile above, its
//     stresses stored with plain stores so they stay in L2), then the item
//     counts itself done for plane p;
//   * velocity half-step of the same tile at plane m = p - WAVE_LAG, after
//     the stresses of planes m-2 .. m+2 are done everywhere: those are all
//     the stresses the velocity loops read (x/y neighbours at plane m, z
//     neighbours of the tile's own columns), and all the stress updates that
//     read the old velocities of plane m.
// The items waited for have lower tickets, so they were claimed by CTAs that
// are running or done and whose stress half-steps wait for nothing: every
// wait ends.  The waits are still bounded (WAVE_SPIN polls of 32-ns sleeps
// scaled by the runtime limit); a wait that runs out raises the solver's
// error word and skips the tile.  Velocity-loop reads of stresses go through
// the coherent path (they were written in this launch); the stresses written
// here and read back a few planes later come from L2, so the step moves each
// array to or from DRAM about once: the 46 words per interior cell of the
// whole step, against 55 for the two-kernel step (stresses written and read
// back, velocities read twice).
constexpr int WAVE_LAG = 4;  // default lag

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// wait until every tile of planes q0..q1 has finished its stress half-step
__device__ __forceinline__ bool wave_wait(const int* done, int q0, int q1, int need, int limit) {
    for (int q = q0; q <= q1; ++q) {
        int it = 0;
        while (ld_acquire(done + q) < need) {
            if (++it > limit) return false;
            __nanosleep(32);
        }
    }
    return true;
}

struct WaveGeom {
    int gxt, gyt, tpp;  // tiles per row, tile rows, tiles per plane
    int lag;            // velocity plane = stress plane - lag (>= 3)
};

// L2 prefetch: the stress inputs of the item `ahead` tickets later, and the
// velocity-phase inputs of this item that nothing has pulled into L2 yet
// (density of plane m+1, and on shell tiles the velocity-loop memories and
// the CPML coefficients of plane m)
__device__ __forceinline__ void wave_prefetch(const S3Args<float>& A, const WaveGeom& G, int t_ahead, int m, int tx,
                                              int ty, int tid) {
    const int nz = A.nz;
    const int pa = t_ahead / G.tpp, ra = t_ahead - pa * G.tpp, tya = ra / G.gxt, txa = ra - tya * G.gxt;
    if (pa >= 1 && pa <= nz - 2) {
        const size_t lin = (size_t)txa + (size_t)G.gxt * ((size_t)tya + (size_t)G.gyt * pa);
        if (tid < NCOEF * NT / 32) pf_l2(A.packed + lin * (NCOEF * NT) + tid * 32);
        pf_tile_rows(A.f, 9, txa, tya, pa, A.nx, A.ny, tid, NT);
        if (!tile_in_box(A.box, txa, tya, pa, A.nx, A.ny)) {
            pf_tile_rows(A.mem, 36, txa, tya, pa, A.nx, A.ny, tid, NT);
            pf_tile_rows(A.cpml, 6, txa, tya, pa, A.nx, A.ny, tid, NT);
        }
    }
    if (m >= 0 && m < nz) {
        if (m + 1 < nz) pf_tile_rows(&A.rho, 1, tx, ty, m + 1, A.nx, A.ny, tid, NT);
        if (!tile_in_box(A.box, tx, ty, m, A.nx, A.ny)) {
            pf_tile_rows(A.mem + 36, 9, tx, ty, m, A.nx, A.ny, tid, NT);
            pf_tile_rows(A.cpml, 6, tx, ty, m, A.nx, A.ny, tid, NT);
        }
    }
}

__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add(int* p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Persistent form: every CTA loops over tickets.  Per item, after the stress
// tile is computed (its shared-memory inputs consumed), the CTA claims its
// next ticket and starts that item's stress copies into the same shared
// memory before it runs the current item's velocity half-step, so the
// coefficient and field stream from DRAM continues while the velocity tile
// works from L2.  The plane counters of a velocity tile are polled by five
// lanes at once.  The deadlock argument of the one-item form holds: the
// owner of the lowest unfinished stress item is either computing it or
// waiting for planes whose items all hold lower tickets, so it never waits
// on itself or on a later item.
// Per-warp norm contribution of the velocity tile into the CTA's running
// maxima (shared memory): FP32 squares as bit patterns (non-negative floats
// order like them, inf and NaN above all finite values), and for a warp with
// a square at or above 3e38 the exact FP64 norms of its cells.
template <typename FA, typename FB>
__device__ __forceinline__ void warp_norm2(float sa, float sb, FA exa, FB exb, unsigned* shu,
                                           unsigned long long* shd) {
    const unsigned ua = __reduce_max_sync(0xffffffffu, __float_as_uint(sa));
    const unsigned ub = __reduce_max_sync(0xffffffffu, __float_as_uint(sb));
    const unsigned big = __float_as_uint(3.0e38f);
    const int lane = threadIdx.x & 31;
    if (ua >= big || ub >= big) {
        double a = exa(), b = exb();
        for (int o = 16; o > 0; o >>= 1) {
            a = nanmax(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = nanmax(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
        if (lane == 0) {
            atomicMax(shd, (unsigned long long)__double_as_longlong(a));
            atomicMax(shd + 1, (unsigned long long)__double_as_longlong(b));
        }
    } else if (lane == 0) {
        atomicMax(shu, ua);
        atomicMax(shu + 1, ub);
    }
}

// Persistent form: every CTA loops over tickets, and no CTA-wide barrier
// sits in the loop.  Per item:
//   * each warp computes its rows of the stress tile from the staged copies
//     and arrives on `freed` once its stores are issued;
//   * warp 0 waits for all eight arrivals, counts the tile done for plane p,
//     claims the next ticket (published through the `ticket` barrier) and
//     starts the next item's copies into the same shared memory, so the DRAM
//     stream goes on while the velocity tile runs;
//   * each warp polls the five plane counters its velocity rows need, runs
//     its rows of the velocity tile from L2, folds its norms into the CTA's
//     running maxima, then reads the next ticket.
// Norm maxima go to the step's slots once, when the CTA runs out of work.
// Deadlock freedom is the one-item argument: the owner of the lowest
// unfinished stress item is either computing it or waiting for planes whose
// items all hold lower tickets.
template <int MINB>
__global__ void __launch_bounds__(NT, MINB) s3w_step(S3Args<float> A, StepInfo si, const __grid_constant__ S3XMaps M,
                                                     WaveGeom G, int total) {
    extern __shared__ __align__(128) float sm[];
    __shared__ __align__(8) unsigned long long bar, freed, ticket_bar;
    __shared__ int s_ticket[2];
    __shared__ unsigned s_nu[2];
    __shared__ unsigned long long s_nd[2];
    const int tid = threadIdx.y * BX + threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    int* ctl = A.wave_ctl;
    int* done = ctl + WAVE_DONE0;
    const int nx = A.nx, ny = A.ny, nz = A.nz, lag = G.lag;
    auto decode = [&](int t, int& p, int& tx, int& ty) {
        p = t / G.tpp;
        const int r = t - p * G.tpp;
        ty = r / G.gxt;
        tx = r - ty * G.gxt;
    };
    auto has_stress = [&](int t) { return t < total && t / G.tpp >= 1 && t / G.tpp <= nz - 2; };
    // arm the copy barrier's next phase and start item t's copies (warp 0)
    auto start_copies = [&](int t) {
        int p, tx, ty;
        decode(t, p, tx, ty);
        if (lane == 0) mbar_expect_tx(&bar, XS_BYTES + (unsigned)probe_bytes(A, tx, ty, p));
        __syncwarp();
        stress_copies_issue(A, M, sm, &bar, tid, tx * BX, ty * BY, p,
                            (size_t)tx + (size_t)G.gxt * ((size_t)ty + (size_t)G.gyt * p));
    };
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_init(&freed, NT / 32);
        mbar_init(&ticket_bar, 1);
        s_ticket[0] = atomicAdd(ctl, 1);
        s_nu[0] = s_nu[1] = 0u;
        s_nd[0] = s_nd[1] = 0ull;
    }
    __syncthreads();
    int t = s_ticket[0];
    if (has_stress(t) && warp == 0) start_copies(t);
    unsigned phase = 0;  // parity of the copy barrier's pending phase
    const int it = *si.step;
    for (int iter = 0; t < total; ++iter) {
        int p, tx, ty;
        decode(t, p, tx, ty);
        const int x0 = tx * BX, y0 = ty * BY;
        const int m = p - lag;
        if (A.prefetch > 0) wave_prefetch(A, G, t + A.prefetch, m, tx, ty, tid);
        // ---- stress half-step of plane p (each warp: its row of the tile)
        const bool st = has_stress(t);
        if (st) {
            const int probe = probe_bytes(A, tx, ty, p);
            if (lean_stress_tile(A, x0, y0, p)) staged_tile<true, false>(A, sm, &bar, tid, x0, y0, p, probe, phase);
            else staged_tile<false, false>(A, sm, &bar, tid, x0, y0, p, probe, phase);
            phase ^= 1u;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&freed);  // this warp's reads of the staging buffer and its stores are done
        if (warp == 0) {
            mbar_wait_bounded(&freed, iter & 1, WAIT_LAND);
            int tn = 0;
            if (lane == 0) {
                if (st) red_release_add(done + p, 1);
                tn = atomicAdd(ctl, 1);
                s_ticket[iter & 1] = tn;
                mbar_arrive(&ticket_bar);
            }
            tn = __shfl_sync(0xffffffffu, tn, 0);
            if (has_stress(tn)) {
                // the generic-proxy reads of the tile just computed come before
                // the asynchronous copies that overwrite it
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                start_copies(tn);
            }
        }
        // ---- velocity half-step of plane m (each warp: its row of the tile)
        if (m >= 0 && m < nz) {
            const int q0 = max(1, m - 2), q1 = min(nz - 2, m + 2);
            const int q = q0 + lane;
            // test hook: one item waits for a count no plane reaches
            const int need = G.tpp + ((A.wait_probe > 0 && t == lag * G.tpp) ? 1 : 0);
            bool ok = true;
            if (q <= q1) {
                int n = 0;
                while (ld_relaxed(done + q) < need) {
                    if (++n > A.wait_limit) { ok = false; break; }
                    __nanosleep(32);
                }
                // the lane that saw the count orders the warp's later reads
                // after the stores the count releases
                asm volatile("fence.acq_rel.gpu;" ::: "memory");
            }
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                if (lane == 0 && A.err) atomicExch(A.err, 1);
            } else {
                const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
                float vsq = 0.f, ssq = 0.f, w[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (lean_tile(A, x0, y0, m, true)) velocity_cell<true, LD_CA>(A, it, gx, gy, m, vsq, ssq, w);
                else if (gx < nx && gy < ny) velocity_cell<false, LD_CA>(A, it, gx, gy, m, vsq, ssq, w);
                warp_norm2(
                    vsq, ssq, [&] { return sqrt((double)w[0] * w[0] + (double)w[1] * w[1] + (double)w[2] * w[2]); },
                    [&] {
                        const double s1 = w[3], s2 = w[4], s3 = w[5], s4 = w[6], s5 = w[7], s6 = w[8];
                        return sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6));
                    },
                    s_nu, s_nd);
            }
        }
        // the next ticket (published by warp 0 once every warp had arrived)
        mbar_wait_bounded(&ticket_bar, iter & 1, WAIT_LAND);
        t = s_ticket[iter & 1];
    }
    __syncthreads();
    if (tid == 0) {
        const double vn = nanmax(sqrt((double)__uint_as_float(s_nu[0])), __longlong_as_double((long long)s_nd[0]));
        const double sn = nanmax(sqrt((double)__uint_as_float(s_nu[1])), __longlong_as_double((long long)s_nd[1]));
        const int slot = blockIdx.x % 64;
        atomic_max_nonneg(A.norms_part + slot, vn);
        atomic_max_nonneg(A.norms_part + 64 + slot, sn);
    }
}

using StressFn = void (*)(S3Args<float>);
// variant 2 (4 CTAs/SM) measured fastest on 352^3: 2.99 ms against 3.42 ms
const StressFn kVariants[] = {s3b_stress<2>, s3b_stress<3>, s3b_stress<4>};
const int kMinBlocks[] = {2, 3, 4};
constexpr int NVAR = sizeof(kVariants) / sizeof(kVariants[0]);

dim3 tile_grid(const S3Args<float>& a) { return dim3((a.nx + BX - 1) / BX, (a.ny + BY - 1) / BY, a.nz); }

}  // namespace

size_t seismic3_bulk_bytes(int nx, int ny, int nz) {
    return (size_t)((nx + BX - 1) / BX) * ((ny + BY - 1) / BY) * nz * TILE_BYTES;
}

int seismic3_bulk_variants() { return NVAR; }
int seismic3_bulk_variant_minblocks(int v) { return (v >= 0 && v < NVAR) ? kMinBlocks[v] : 0; }

cudaError_t seismic3_bulk_pack(const S3Args<float>& a, float* packed, cudaStream_t st) {
    s3b_pack<<<tile_grid(a), dim3(BX, BY), 0, st>>>(a, packed);
    return cudaGetLastError();
}

// Tensor maps of the staged kernel; false when the grid does not meet the
// tensor-copy rules (row pitch a multiple of 16 bytes) or the driver entry
// point is missing, in which case the caller keeps the bulk kernel.
bool seismic3_staged_prepare(const S3Args<float>& a, S3XMaps* m) {
    if (a.nx % 4 != 0) return false;
    for (int q = 0; q < 6; ++q)
        if (!seismic3_make_map(&m->sig[q], a.f[3 + q], a.nx, a.ny, a.nz, BX, BY)) return false;
    for (int f = 0; f < 3; ++f) {
        if (!seismic3_make_map(&m->vh[f], a.f[f], a.nx, a.ny, a.nz, VHW, VHH)) return false;
        if (!seismic3_make_map(&m->vp[f], a.f[f], a.nx, a.ny, a.nz, BX, BY)) return false;
    }
    for (const void* fn : {(const void*)s3x_stress<4>, (const void*)s3x_stress<4, false, true>}) {
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)XS_BYTES) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
    }
    return true;
}

void launch_seismic3_staged_stress(const S3Args<float>& a, const S3XMaps& maps, cudaStream_t st) {
    const dim3 grd = tile_grid(a), blk(BX, BY);
    if (a.mat_ids && a.mem_merged) s3x_stress<4, true, true><<<grd, blk, XI_BYTES, st>>>(a, maps);
    else if (a.mat_ids) s3x_stress<4, true><<<grd, blk, XI_BYTES, st>>>(a, maps);
    else if (a.mem_merged) s3x_stress<4, false, true><<<grd, blk, XS_BYTES, st>>>(a, maps);
    else s3x_stress<4><<<grd, blk, XS_BYTES, st>>>(a, maps);
}

int seismic3_wave_prepare(const S3Args<float>& a) {
    if (!a.staged || !a.wave_ctl) return 0;
    if (cudaFuncSetAttribute((const void*)s3w_step<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)XS_BYTES) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per_sm = 0, dev = 0, nsm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)s3w_step<4>, NT, XS_BYTES) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return 0;
    }
    return per_sm * nsm;
}

void launch_seismic3_wave(const S3Args<float>& a, const S3XMaps& maps, const StepInfo& s, cudaStream_t st) {
    WaveGeom G;
    G.gxt = (a.nx + BX - 1) / BX;
    G.gyt = (a.ny + BY - 1) / BY;
    G.tpp = G.gxt * G.gyt;
    G.lag = a.wave_lag >= 3 ? a.wave_lag : WAVE_LAG;
    const int items = G.tpp * (a.nz + G.lag);
    // one CTA per resident slot (4 per SM); each loops over tickets
    const int grid = std::min(items, a.wave_ctas > 0 ? a.wave_ctas : items);
    s3w_step<4><<<grid, dim3(BX, BY), XS_BYTES, st>>>(a, s, maps, G, items);
}

void launch_seismic3_bulk_stress(const S3Args<float>& a, int variant, cudaStream_t st) {
    const StressFn fn = kVariants[(variant >= 0 && variant < NVAR) ? variant : 0];
    fn<<<tile_grid(a), dim3(BX, BY), TILE_BYTES, st>>>(a);
}
