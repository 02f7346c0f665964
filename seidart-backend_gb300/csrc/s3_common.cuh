// s3_common.cuh -- device helpers shared by the FP32 one-cell-per-thread 3D
// elastic kernels (seismic3_cell.cu, seismic3_bulk.cu): clamped stencil
// offsets, the C-PML memory update of the stress loops
// (src/fortran/cpmlfdtd.f08:1761-1992) and the anisotropic stress update, plus
// the mbarrier / bulk-copy primitives of the shared-memory staged kernels.
#pragma once
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"

namespace s3 {

__device__ __forceinline__ int cl(int v, int lo, int hi) { return min(max(v, lo), hi); }

struct CpmlC {
    float b, a, k;
};
__device__ __forceinline__ CpmlC cpml_at(const S3Args<float>& A, size_t c, bool half) {
    return half ? CpmlC{__ldcs(A.cpml[5] + c), __ldcs(A.cpml[3] + c), __ldcs(A.cpml[1] + c)}
                : CpmlC{__ldcs(A.cpml[4] + c), __ldcs(A.cpml[2] + c), __ldcs(A.cpml[0] + c)};
}
__device__ __forceinline__ float cpml_apply(float* m, size_t c, const CpmlC& p, float d) {
    const float mv = p.b * m[c] + p.a * d;
    m[c] = mv;
    return d * p.k + mv;
}
// The C-PML step of stress loop L (1: normal stresses, 2: sigma_xy,
// 3: sigma_xz, 4: sigma_yz; memory slots 9(L-1)..9L-1) in three parts, so a
// kernel can issue the loads of two loops before the stores of either:
// cpml_load reads the nine memories, cpml_update advances them and rescales
// the loop's nine derivatives, cpml_store writes them back.
struct CpmlPair {
    CpmlC h, f;  // half-grid and full-grid coefficient triples of the cell
};
__device__ __forceinline__ CpmlPair cpml_both(const S3Args<float>& A, size_t c) {
    return CpmlPair{cpml_at(A, c, true), cpml_at(A, c, false)};
}
// place of cell (x, y, k) in the tile-packed byte layouts: tile (x/32, y/8,
// k) of the 32 x 8 tile grid, then (y % 8) * 32 + x % 32 within the tile
__device__ __forceinline__ size_t tile_byte(int nx, int ny, int x, int y, int k) {
    const int gx = (nx + 31) >> 5, gy = (ny + 7) >> 3;
    return (((size_t)k * gy + (y >> 3)) * gx + (x >> 5)) * 256 + ((y & 7) << 5) + (x & 31);
}
// both C-PML coefficient triples of cell c = (x, y, k): from the indexed
// table when the solver found one (the same FP32 values), else the grids
__device__ __forceinline__ CpmlPair cpml_pair_at(const S3Args<float>& A, size_t c, int x, int y, int k) {
    if (A.cpml_ids) {
        const float* T = A.cpml_tab + 6 * __ldg(A.cpml_ids + tile_byte(A.nx, A.ny, x, y, k));
        return CpmlPair{CpmlC{__ldg(T + 5), __ldg(T + 3), __ldg(T + 1)}, CpmlC{__ldg(T + 4), __ldg(T + 2), __ldg(T)}};
    }
    return cpml_both(A, c);
}
// L2 prefetch of the C-PML coefficients of tile (tx, ty, k) of the 32 x 8
// grid: its 256 index bytes, or the six grids' rows
__device__ __forceinline__ void pf_cpml_tile(const S3Args<float>& A, int tx, int ty, int k, int tid, int nthreads);
template <int L>
__device__ __forceinline__ void cpml_load(const S3Args<float>& A, size_t c, float (&m)[9]) {
    float* const* M = A.mem + 9 * (L - 1);
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = M[q][c];
}
template <int L>
__device__ __forceinline__ void cpml_store(const S3Args<float>& A, size_t c, const float (&m)[9]) {
    float* const* M = A.mem + 9 * (L - 1);
#pragma unroll
    for (int q = 0; q < 9; ++q) M[q][c] = m[q];
}
template <int L>
__device__ __forceinline__ void cpml_update(const CpmlPair& P, float (&m)[9], float (&gx)[3], float (&gy)[3],
                                            float (&gz)[3]) {
    constexpr bool xh = (L == 1 || L == 4), yh = (L == 2 || L == 4), zh = (L != 1);
    const CpmlC px = xh ? P.h : P.f, py = yh ? P.h : P.f, pz = zh ? P.h : P.f;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        m[3 * f] = px.b * m[3 * f] + px.a * gx[f];
        gx[f] = gx[f] * px.k + m[3 * f];
        m[3 * f + 1] = py.b * m[3 * f + 1] + py.a * gy[f];
        gy[f] = gy[f] * py.k + m[3 * f + 1];
        // loop 2 advances memory_dvx_dz2 but sigma_xy uses the raw dvx_dz
        // (reference quirk, cpmlfdtd.f08:1855-1866)
        m[3 * f + 2] = pz.b * m[3 * f + 2] + pz.a * gz[f];
        if (!(L == 2 && f == 0)) gz[f] = gz[f] * pz.k + m[3 * f + 2];
    }
}

// C-PML correction of the nine derivatives of stress loop L, loads first
template <int L>
__device__ __forceinline__ void loop_cpml(const S3Args<float>& A, size_t c, float (&gx)[3], float (&gy)[3],
                                          float (&gz)[3]) {
    const CpmlPair P = cpml_both(A, c);
    // all nine memories are loaded before the first store: a store to one
    // memory array would otherwise hold the next array's load behind it (the
    // compiler cannot rule out aliasing), one DRAM round trip per memory
    float m[9];
    cpml_load<L>(A, c, m);
    cpml_update<L>(P, m, gx, gy, gz);
    cpml_store<L>(A, c, m);
}

// sigma_new = (sigma_old + dt * sum_j C_ij e_j) / (1 + gamma dt); C read
// through the accessor so the coefficients may come from registers or smem
template <typename CF>
__device__ __forceinline__ float stress_new(CF C, float so, float gm, int c1, int c2, int c3, int c4, int c5, int c6,
                                            float dt, const float (&gx)[3], const float (&gy)[3],
                                            const float (&gz)[3]) {
    const float acc = C(c1) * gx[0] + C(c2) * gy[1] + C(c3) * gz[2] + C(c4) * (gz[1] + gy[2]) +
                      C(c5) * (gz[0] + gx[2]) + C(c6) * (gx[1] + gy[0]);
    return (so + acc * dt) * gm;
}

// ------------------------------------------------ mbarrier + bulk copies
__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// plain arrival (release at CTA scope) on a barrier counting warps or threads
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
// complete `bytes` of the barrier's pending transaction count from this
// thread (the test hook's stand-in for bytes that never arrive)
__device__ __forceinline__ void mbar_complete_tx(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
// bounded wait: false when the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* b, unsigned parity, int limit) {
    for (int it = 0; it < limit; ++it)
        if (mbar_try_wait(b, parity)) return true;
    return false;
}
// contiguous global -> shared copy (both 16-byte aligned, bytes % 16 == 0)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}

// 3D tensor-tile global -> shared copy (TMA); x * 4 must be a multiple of 16
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, int x, int y, int z,
                                          unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            saddr(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
        : "memory");
}

// L2 eviction policy for read-once streams: lines they bring in go first,
// so data another CTA reads again (velocity planes) stays longer
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void bulk_g2s_hint(void* dst, const void* src, unsigned bytes, unsigned long long* bar,
                                              uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
            "r"(saddr(dst)),
        "l"(src), "r"(bytes), "r"(saddr(bar)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ void tma_load3_hint(void* dst, const CUtensorMap* map, int x, int y, int z,
                                               unsigned long long* bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, "
        "%3, %4}], [%5], %6;" ::"r"(saddr(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(saddr(bar)), "l"(pol)
        : "memory");
}

// ------------------------------------------------------ L2 prefetch
__device__ __forceinline__ void pf_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Prefetch into L2 the rows of one 32 x 8 tile (tile indices tx, ty, plane k)
// of `narr` arrays; row segment q of array q / 8 is covered by its first and
// last element (a 128-byte segment spans at most two lines).  Work is spread
// over the CTA's threads (tid of nthreads).
__device__ __forceinline__ void pf_tile_rows(const float* const* arr, int narr, int tx, int ty, int k, int nx, int ny,
                                             int tid, int nthreads) {
    const int x0 = tx * 32, x1 = min(x0 + 31, nx - 1);
    for (int q = tid; q < narr * 8; q += nthreads) {
        const int y = ty * 8 + (q & 7);
        if (y >= ny) continue;
        const float* row = arr[q >> 3] + ((size_t)k * ny + y) * nx;
        pf_l2(row + x0);
        pf_l2(row + x1);
    }
}

__device__ __forceinline__ void pf_cpml_tile(const S3Args<float>& A, int tx, int ty, int k, int tid, int nthreads) {
    if (A.cpml_ids) {
        const int gx = (A.nx + 31) >> 5, gy = (A.ny + 7) >> 3;
        if (tid < 2) pf_l2(A.cpml_ids + (((size_t)k * gy + ty) * gx + tx) * 256 + tid * 128);
    } else {
        pf_tile_rows(A.cpml, 6, tx, ty, k, A.nx, A.ny, tid, nthreads);
    }
}

// The tile `d` (x, y, z offsets of a distance in launch order) after this
// CTA's on the launch grid, with carries; false past the last tile.  The host
// splits the distance once, so no thread divides.
__device__ __forceinline__ bool tile_ahead(const int (&d)[3], int& tx, int& ty, int& k) {
    int x = (int)blockIdx.x + d[0], y = (int)blockIdx.y + d[1], z = (int)blockIdx.z + d[2];
    if (x >= (int)gridDim.x) { x -= gridDim.x; ++y; }
    if (y >= (int)gridDim.y) { y -= gridDim.y; ++z; }
    if (z >= (int)gridDim.z) return false;
    tx = x; ty = y; k = z;
    return true;
}

// true when the 32 x 8 tile (tx, ty, k) lies inside the inert interior box,
// where no CPML memory or coefficient is touched
__device__ __forceinline__ bool tile_in_box(const BoxH& b, int tx, int ty, int k, int nx, int ny) {
    const int x0 = tx * 32, x1 = min(x0 + 32, nx), y0 = ty * 8, y1 = min(y0 + 8, ny);
    return x0 >= b.i0 && x1 <= b.i1 && y0 >= b.j0 && y1 <= b.j1 && k >= b.k0 && k < b.k1;
}

}  // namespace s3
