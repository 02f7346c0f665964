// noalloc.cu -- trace misfit of device-resident traces without any device
// allocation.
//
// Variant of the residual/misfit kernel behind seidart_fwi_gradient
// (residual_loss in adjoint.cu), whose FP64 accumulator lives in memory that
// seidart_fwi_create allocates.  Here the accumulators are a fixed,
// file-scope device array: one FP64 slot per trace column (at most
// SEIDART_NOALLOC_MAX_TRACES) plus one slot for the total, 64 KiB in all.
// The only CUDA runtime calls are a symbol-address lookup (first call on
// each device), one memset, two kernel launches, device-to-host copies of
// the results and a stream synchronize: no cudaMalloc, cudaFree or library
// routine that allocates.
//
// What must start at zero: the ntraces per-trace accumulators; every call
// clears them with cudaMemsetAsync on the caller's stream before its first
// kernel.  The total slot is written, not accumulated.
// Calls that overlap on one device (two host threads, or two streams
// without ordering between them) share the accumulators and corrupt each
// other's results: callers serialise calls per device.
// The device address of the array and the SM count are looked up once per
// device and kept for the life of the process; cudaDeviceReset between
// calls is not supported (it unloads the module, and the kept address would
// then point at freed memory).
#include <cuda_runtime.h>
#include <stdio.h>

#include <atomic>

#include "../../include/seidart_gpu.h"

namespace {

constexpr int MAXT = SEIDART_NOALLOC_MAX_TRACES;
constexpr int TB = 256;
constexpr int MAX_DEVICES = 64;

// [0, MAXT): per-trace sums; [MAXT]: total
static __device__ __align__(256) double g_misfit_scratch[MAXT + 32];

std::atomic<double*> g_scratch_ptr[MAX_DEVICES];
std::atomic<int> g_sm_count[MAX_DEVICES];

}  // namespace

extern "C" int seidart_internal_set_error(int code, const char* msg);

namespace {

int nerr(int code, const char* msg) { return seidart_internal_set_error(code, msg); }

// columns t = blockIdx.x*TB + threadIdx.x; each block sums a slab of steps
__global__ void __launch_bounds__(TB) misfit_partial(const float* __restrict__ syn, const float* __restrict__ obs,
                                                     float* __restrict__ res, int nsteps, int ntraces,
                                                     int steps_per_block, double* acc) {
    const int t = blockIdx.x * TB + threadIdx.x;
    if (t >= ntraces) return;
    const int s0 = blockIdx.y * steps_per_block;
    const int s1 = min(nsteps, s0 + steps_per_block);
    double a = 0.0;
    for (int s = s0; s < s1; ++s) {
        const size_t q = (size_t)s * ntraces + t;
        const float r = syn[q] - obs[q];
        if (res) res[q] = r;
        a += (double)r * (double)r;
    }
    if (s1 > s0) atomicAdd(acc + t, 0.5 * a);
}

// total = sum of the per-trace sums, in a fixed order
__global__ void __launch_bounds__(TB) misfit_total(int ntraces, double* acc) {
    __shared__ double red[TB];
    double a = 0.0;
    for (int t = threadIdx.x; t < ntraces; t += TB) a += acc[t];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int w = TB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) acc[MAXT] = red[0];
}

}  // namespace

extern "C" {

int seidart_trace_misfit_noalloc(const float* syn, const float* obs, float* residual, int nsteps, int ntraces,
                                 double* misfit, double* total, void* stream) {
    if (!syn || !obs || !total) return nerr(SEIDART_ERR_ARG, "syn, obs and total must not be NULL");
    if (nsteps < 1 || ntraces < 1) return nerr(SEIDART_ERR_ARG, "nsteps and ntraces must be positive");
    if (ntraces > MAXT) {
        char m[160];
        snprintf(m, sizeof m, "ntraces = %d exceeds the fixed scratch of SEIDART_NOALLOC_MAX_TRACES = %d trace columns",
                 ntraces, MAXT);
        return nerr(SEIDART_ERR_ARG, m);
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
        return nerr(SEIDART_ERR_CUDA, "no current CUDA device");
    double* acc = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!acc) {
        // first call on this device (the current one): look the array up
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_misfit_scratch);
        if (e != cudaSuccess || !p) return nerr(SEIDART_ERR_CUDA, cudaGetErrorString(e));
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
            return nerr(SEIDART_ERR_CUDA, "cannot read the SM count of the current device");
        g_sm_count[dev].store(sms, std::memory_order_relaxed);
        acc = (double*)p;
        g_scratch_ptr[dev].store(acc, std::memory_order_release);
    }
    const int sms = g_sm_count[dev].load(std::memory_order_relaxed);
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(acc, 0, sizeof(double) * ntraces, st) != cudaSuccess)
        return nerr(SEIDART_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    const int gx = (ntraces + TB - 1) / TB;
    const int want_y = (4 * sms + gx - 1) / gx;  // about four CTAs per SM in all
    const int spb = (nsteps + want_y - 1) / want_y;
    const int gy = (nsteps + spb - 1) / spb;
    misfit_partial<<<dim3(gx, gy), TB, 0, st>>>(syn, obs, residual, nsteps, ntraces, spb, acc);
    misfit_total<<<1, TB, 0, st>>>(ntraces, acc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return nerr(SEIDART_ERR_CUDA, cudaGetErrorString(e));
    if (cudaMemcpyAsync(total, acc + MAXT, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        (misfit && cudaMemcpyAsync(misfit, acc, sizeof(double) * ntraces, cudaMemcpyDeviceToHost, st) != cudaSuccess))
        return nerr(SEIDART_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nerr(SEIDART_ERR_CUDA, cudaGetErrorString(e));
    return SEIDART_OK;
}

}  // extern "C"
