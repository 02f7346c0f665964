// common.cuh -- shared device helpers for the CPML-FDTD kernels.
//
// Each solver .cu file is compiled three times: with SEIDART_REAL=double and
// --fmad=false (the drop-in FP64 path, which keeps the reference's expression
// trees so results are reproducible operation by operation), with
// SEIDART_REAL=double, SEIDART_FAST64 and FMA contraction (FP64 fields with
// the fast path's arithmetic: host-side reciprocals instead of divisions,
// contracted multiply-adds, FP64 norms), and with SEIDART_REAL=float and FMA
// contraction (the fast FP32 path).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef SEIDART_REAL
#define SEIDART_REAL double
#endif
typedef SEIDART_REAL real;

#define SD_CAT2(a, b) a##b
#define SD_CAT(a, b) SD_CAT2(a, b)
// SD_EXACT: the reference's divisions and operation order; SD_F32: FP32
// storage and FP32 norm reductions
#if defined(SEIDART_FP32)
#define SD_SUFFIX _f32
#define SD_EXACT 0
#define SD_F32 1
#elif defined(SEIDART_FAST64)
#define SD_SUFFIX _f64x
#define SD_EXACT 0
#define SD_F32 0
#else
#define SD_SUFFIX _f64
#define SD_EXACT 1
#define SD_F32 0
#endif
// launcher names carry the precision suffix so both builds link into one library
#define SD_NAME(n) SD_CAT(n, SD_SUFFIX)

// Axis-aligned box [lo, hi) per axis (0-based) inside which the CPML
// coefficients are inert (acoef = acoef_half = 0, kappa = kappa_half = 1):
// there the memory variables stay zero and the derivative passes through
// unchanged, so kernels skip the CPML arithmetic and its memory traffic.
struct Box {
    int i0, i1, j0, j1, k0, k1;
};

__device__ __forceinline__ bool in_box2(const Box& b, int i, int k) {
    return i >= b.i0 && i < b.i1 && k >= b.k0 && k < b.k1;
}
__device__ __forceinline__ bool in_box3(const Box& b, int i, int j, int k) {
    return i >= b.i0 && i < b.i1 && j >= b.j0 && j < b.j1 && k >= b.k0 && k < b.k1;
}

// scalar_mean, src/fortran/averaging.f08:5-25 (FP64 path: same operations)
__device__ __forceinline__ double scalar_mean_d(double a, double b, int code) {
    switch (code) {
    case 1: return 2.0 * a * b / (a + b);
    case 2: return sqrt(a * b);
    case 3: return 0.5 * (a + b);
    default: return a;
    }
}
// FP32 path: reciprocal of the face density (buoyancy) directly
__device__ __forceinline__ float inv_mean_f(float a, float b, int code) {
    switch (code) {
    case 1: return __fdividef(a + b, 2.0f * a * b);
    case 2: return rsqrtf(a * b);
    case 3: return __fdividef(2.0f, a + b);
    default: return __frcp_rn(a);
    }
}
// fast FP64 path: the same reciprocal forms in FP64 (one division per face)
__device__ __forceinline__ double inv_mean_f(double a, double b, int code) {
    switch (code) {
    case 1: return (a + b) / (2.0 * a * b);
    case 2: return 1.0 / sqrt(a * b);
    case 3: return 2.0 / (a + b);
    default: return 1.0 / a;
    }
}

// Max-norm accumulation: non-negative doubles order like their bit patterns,
// so an unsigned 64-bit atomicMax gives the exact maximum.  NaN (bit pattern
// above +inf) also wins, which flags a NaN blow-up as unstable.
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(addr),
              static_cast<unsigned long long>(__double_as_longlong(v)));
}

// max that lets a NaN win (fmax would drop it)
__device__ __forceinline__ double nanmax(double a, double b) {
    return (a != a) ? a : ((b != b) ? b : fmax(a, b));
}

__device__ __forceinline__ float nanmaxf(float a, float b) {
    return (a != a) ? a : ((b != b) ? b : fmaxf(a, b));
}

// Block-wide max in FP32 (result valid in warp 0).
template <int NW>
__device__ __forceinline__ float block_maxf(float v, float* sh) {
    for (int o = 16; o > 0; o >>= 1) v = nanmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (lane < NW) ? sh[lane] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) v = nanmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

// Block-wide max of v over NW warps; every thread of the block must call it.
// The result is valid in warp 0.
template <int NW>
__device__ __forceinline__ double block_max(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (lane < NW) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

// Block max of a Euclidean norm for the FP32 kernels: the squared norm `sq`
// is reduced in FP32 and one FP64 square root is taken per block.  If any
// square in the block is not representable in FP32 (or is NaN), the block is
// reduced again from the exact FP64 norms `exact()` so the 1e25 blow-up test
// keeps FP64 semantics.  Every thread of the block must call it (uniform
// control flow); the result is valid in warp 0.
// (only thread 0 takes the FP64 square root; the other threads return 0)
template <int NW, typename F>
__device__ __forceinline__ double block_norm_f32(float sq, F exact, float* shf, double* shd) {
    const int big = __syncthreads_or(!(sq < 3.0e38f));
    const bool t0 = (threadIdx.x | threadIdx.y | threadIdx.z) == 0;
    if (!big) {
        const float m = block_maxf<NW>(sq, shf);
        return t0 ? sqrt((double)m) : 0.0;
    }
    const double m = block_max<NW>(exact(), shd);
    return t0 ? m : 0.0;
}

// Two max-norms of a block at once.  Non-negative FP32 squares order like
// their bit patterns, with inf and NaN above every finite value, so one
// redux.sync max per warp and one barrier give both block maxima.  A block
// whose larger square is not below 3e38 (overflow, inf or NaN) redoes both in
// FP64 through exa()/exb() (uniform branch).  Results are valid on thread 0:
// sqrt of each maximum.  shu: [2][NW] unsigned, shd: [2][NW] double.
template <int NW, typename FA, typename FB>
__device__ __forceinline__ void block_norm2_f32(float sa, float sb, FA exa, FB exb, unsigned* shu, double* shd,
                                                double& na, double& nb) {
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const unsigned ua = __reduce_max_sync(0xffffffffu, __float_as_uint(sa));
    const unsigned ub = __reduce_max_sync(0xffffffffu, __float_as_uint(sb));
    if ((tid & 31) == 0) {
        shu[tid >> 5] = ua;
        shu[NW + (tid >> 5)] = ub;
    }
    __syncthreads();
    unsigned ma = 0u, mb = 0u;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        ma = max(ma, shu[w]);
        mb = max(mb, shu[NW + w]);
    }
    const unsigned big = __float_as_uint(3.0e38f);  // squares at or above it go to FP64
    if (ma >= big || mb >= big) {
        const double a = block_max<NW>(exa(), shd);
        const double b = block_max<NW>(exb(), shd + NW);
        na = a;
        nb = b;
    } else if (tid == 0) {  // FP64 square roots are slow here: thread 0 only
        na = sqrt((double)__uint_as_float(ma));
        nb = sqrt((double)__uint_as_float(mb));
    } else {
        na = nb = 0.0;
    }
}
