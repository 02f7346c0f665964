// solver.cu -- host runtime behind the C ABI (include/seidart_gpu.h).
//
// A SeidartSolver owns, for one model, a single device arena holding the
// model arrays (converted once to the field precision, with FP64-derived
// coefficients such as 1/(1+gamma dt), 1/kappa or the EM tensor inverses),
// the fields, the full-grid CPML memory arrays, the source series, the
// receiver traces and the per-step norms.  Steps run asynchronously on the
// solver's stream; chunks of steps are captured once into a CUDA graph and
// replayed (the step number lives in device memory, so one graph serves
// every starting step).
//
// Host-side coefficient set-up follows the reference formulas statement by
// statement (this file is compiled with -ffp-contract=off so the FP64 values
// match the CPU restatement exactly).
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "../../include/seidart_gpu.h"
#include "host_pool.h"
#include "trace.h"
#include "kernels.h"

// plane-wave set-up (planewave.cu)
int pw_setup(int family, const SeidartDomain* dom, const SeidartSource* src, const SeidartPlaneWave* in,
             const double* const* model, PwDev* out, std::string& why);

namespace {

thread_local std::string g_err;

int set_err(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CUDA_TRY(expr)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return set_err(SEIDART_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(e_)); \
    } while (0)

const double kPi = 3.141592653589793238462643;
const double kEps0 = 8.85418782e-12;
const double kMu0 = 4.0 * kPi * 1.0e-7;  // constants.f08:9

struct Layout {
    int nmodel, nsrc, nfield, nmem, cplx, ncomp;
};
bool layout_of(int fam, Layout* L) {
    switch (fam) {
    case SEIDART_SEISMIC2: *L = {S2_NMODEL, S2_NSRC, S2_NFIELD, S2_NMEM, 0, 2}; return true;
    case SEIDART_SEISMIC25: *L = {SEIDART_NMODEL3, S3_NSRC, S3_NFIELD, S25_NMEM, 1, 3}; return true;
    case SEIDART_SEISMIC3: *L = {SEIDART_NMODEL3, S3_NSRC, S3_NFIELD, S3_NMEM, 0, 3}; return true;
    case SEIDART_ELECTROMAG2: *L = {E2_NMODEL, E2_NSRC, E2_NFIELD, E2_NMEM, 0, 2}; return true;
    case SEIDART_ELECTROMAG25: *L = {E25_NMODEL, E25_NSRC, E25_NFIELD, E25_NMEM, 1, 3}; return true;
    case SEIDART_ELECTROMAG3: *L = {E3_NMODEL, E3_NSRC, E3_NFIELD, E3_NMEM, 0, 3}; return true;
    default: return false;
    }
}

// CPML slot offsets inside each family's model list (kappa, kappa_half,
// acoef, acoef_half, bcoef, bcoef_half are always consecutive).
int cpml_slot(int fam) {
    switch (fam) {
    case SEIDART_SEISMIC2: return S2_KAPPA;
    case SEIDART_ELECTROMAG2: return E2_KAPPA;
    case SEIDART_ELECTROMAG25: return E25_KAPPA;
    case SEIDART_ELECTROMAG3: return E3_KAPPA;
    default: return SEIDART_KAPPA3;
    }
}

// array_averaging2d, averaging.f08:27-80 (in place, ascending: '+i'/'+j'
// are running averages)
double scalar_mean_h(double a, double b, int code) {
    switch (code) {
    case 1: return 2.0 * a * b / (a + b);
    case 2: return sqrt(a * b);
    case 3: return 0.5 * (a + b);
    default: return a;
    }
}
void averaging2d(double* a, int ni, int nj, int code, int dir) {
    auto ix = [ni](int i, int j) { return (size_t)(i - 1) + (size_t)ni * (size_t)(j - 1); };
    switch (dir) {
    case 0: for (int j = 1; j <= nj; ++j) for (int i = 2; i <= ni; ++i) a[ix(i, j)] = scalar_mean_h(a[ix(i, j)], a[ix(i - 1, j)], code); break;
    case 1: for (int j = 1; j <= nj; ++j) for (int i = 1; i <= ni - 1; ++i) a[ix(i, j)] = scalar_mean_h(a[ix(i, j)], a[ix(i + 1, j)], code); break;
    case 2: for (int j = 2; j <= nj; ++j) for (int i = 1; i <= ni; ++i) a[ix(i, j)] = scalar_mean_h(a[ix(i, j)], a[ix(i, j - 1)], code); break;
    default: for (int j = 1; j <= nj - 1; ++j) for (int i = 1; i <= ni; ++i) a[ix(i, j)] = scalar_mean_h(a[ix(i, j)], a[ix(i, j + 1)], code); break;
    }
}

// zero the six faces of a 3D grid (electromag3's H fields, zeroed lazily)
template <typename T>
__global__ void zero_faces3d(T* f, int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / ((size_t)nx * ny));
        if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1) f[c] = 0;
    }
}

template <typename T>
__global__ void zero_ring2d(T* f, int nx, int nz, int ncomp_per_cell) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int per = 2 * nx + 2 * nz;
    if (t >= per) return;
    int i, k;
    if (t < nx) { i = t; k = 0; }
    else if (t < 2 * nx) { i = t - nx; k = nz - 1; }
    else if (t < 2 * nx + nz) { i = 0; k = t - 2 * nx; }
    else { i = nx - 1; k = t - 2 * nx - nz; }
    const size_t c = (size_t)i + (size_t)nx * k;
    for (int q = 0; q < ncomp_per_cell; ++q) f[c * ncomp_per_cell + q] = 0;
}

}  // namespace

struct SeidartSolver {
    int family = 0, precision = 0, density = 1;
    SeidartDomain dom{};
    SeidartSource src{};
    Layout L{};
    size_t ncell = 0, esize = 8;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    char* arena = nullptr;
    size_t arena_bytes = 0, arena_used = 0;
    std::vector<void*> fields, mem;
    int* step_dev = nullptr;
    int* rec_dev = nullptr;
    int nrec = 0;
    void* traces = nullptr;
    double* norms = nullptr;
    double* norms_part = nullptr;  // per-step partial maxima of the FP32 3D kernels
    // FP32 3D kernels per half-step (S3K_BULK, S3K_CELL, S3K_ZMARCH, S3K_TMA);
    // the environment variables SEIDART_S3_STRESS / SEIDART_S3_VELOCITY
    // (bulk | cell | zmarch | tma) and SEIDART_S3_TMA / SEIDART_S3_BULK
    // (variant numbers) override them
    int s3_stress_kind = S3K_BULK, s3_velocity_kind = S3K_CELL;
    float* s3_packed = nullptr;  // tile-packed coefficients of the bulk stress kernel
    double* stage = nullptr;     // FP64 staging buffer for on-device precision conversion (FP32 solvers)
    size_t stage_n = 0;          // its capacity in doubles
    float* pin = nullptr;        // pinned host double buffer of FP32 read-backs (2 x kPinChunk floats)
    cudaEvent_t pin_ev[2] = {nullptr, nullptr};
    S3XMaps s3_staged{};         // tensor maps of the staged stress kernel (when s3f.staged is set)
    unsigned char* s3_mat_ids = nullptr;  // material-indexed model: one byte per cell, tile-packed
    float* s3_mat_tab = nullptr;          // and the [S3_MAXMAT][27] table of FP32 coefficient tuples
    int s3_nmat = 0;                      // materials of the indexed layout (0: per-cell arrays)
    unsigned char* s3_cpml_ids = nullptr; // indexed C-PML coefficients: one byte per cell, tile-packed
    float* s3_cpml_tab = nullptr;         // and the [S3_MAXCPML][6] table
    int s3_ncpml = 0;                     // C-PML tuples of the indexed layout (0: the six grids)
    bool s3_tma = false;  // TMA-fed stress kernel prepared (grid meets the TMA rules)
    int s3_tma_variant = 0;
    S3Maps s3_maps;       // its tensor maps
    int* err_dev = nullptr;  // error word raised by bounded device waits
    int* wave_ctl = nullptr; // FP32 3D fused step: work ticket and per-plane counters (arena)
    int wave_n = 0;
    int nnorm = 1;
    int steps_done = 0;
    int stress_src = 0;
    BoxH box{};
    long long launches = 0;
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
    int graph_len[2] = {0, 0};
    bool graphs_ok = true;
    // precision-specific launch argument blocks
    S2Args<double> s2d; S2Args<float> s2f;
    E2Args<double> e2d; E2Args<float> e2f;
    S25Args<double> s25d; S25Args<float> s25f;
    E25Args<double> e25d; E25Args<float> e25f;
    E3Args<double> e3d; E3Args<float> e3f;
    S3Args<double> s3d; S3Args<float> s3f;

    void* carve(size_t bytes) {
        const size_t off = (arena_used + 255) & ~(size_t)255;
        arena_used = off + bytes;
        return arena ? arena + off : nullptr;
    }
};

namespace {

// Upload n values of `h` (FP64) as T into device memory d.
// FP64 host data -> FP32 device arrays through an FP64 staging buffer and a
// conversion kernel (the FP64 arithmetic of the derived forms rounded per
// operation, as the host would compute it), so set-up and read-back do not
// convert element by element on one host core.
// mode 0: x;  1: 1/(1 + x dt) (attenuation factor);  2: 1/x
__global__ void convert_to_f32(float* __restrict__ d, const double* __restrict__ h, size_t n, int mode, double dt) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        double x = h[q];
        if (mode == 1) x = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(x, dt)));
        else if (mode == 2) x = __ddiv_rn(1.0, x);
        d[q] = __double2float_rn(x);
    }
}
// the same derived forms in place on FP64 arrays (fast FP64 solvers)
__global__ void derive_f64(double* __restrict__ d, size_t n, int mode, double dt) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const double x = d[q];
        d[q] = mode == 1 ? __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(x, dt))) : __ddiv_rn(1.0, x);
    }
}
// The reference's memory q (0..35) of stress loop L = q / 9 + 1 from the
// merged layout of the FP32 staged stress kernel: the slot that holds it
// (its own, or the one the loop shares with another loop for the same
// stencil and coefficients) where loop L updates the cell, zero elsewhere --
// the reference never advances a loop's memory outside the loop's range.
__global__ void s3_unmerge(S3Args<float> a, int q, float* __restrict__ out) {
    const int L = q / 9 + 1, f = (q % 9) / 3, d = q % 3;
    int slot = q;
    if (L == 3 && d == 0) slot = 9 + 3 * f;       // backward x, full: loop 2's
    if (L == 3 && d == 1) slot = 3 * f + 1;       // backward y, full: loop 1's
    if (L == 4 && d == 0) slot = 3 * f;           // forward x, half: loop 1's
    if (L == 4 && d == 1) slot = 9 + 3 * f + 1;   // forward y, half: loop 2's
    if (L == 4 && d == 2) slot = 18 + 3 * f + 2;  // forward z, half: loop 3's
    const float* src = a.mem[slot];
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const size_t n = (size_t)nx * ny * nz;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / ((size_t)nx * ny));
        const bool x14 = i >= 1 && i <= nx - 3, x23 = i >= 2 && i <= nx - 2;
        const bool y13 = j >= 2 && j <= ny - 2, y24 = j >= 1 && j <= ny - 3;
        const bool z12 = k >= 2 && k <= nz - 2, z34 = k >= 1 && k <= nz - 3;
        const bool in = L == 1 ? (x14 && y13 && z12) : L == 2 ? (x23 && y24 && z12)
                      : L == 3 ? (x23 && y13 && z34) : (x14 && y24 && z34);
        out[c] = in ? src[c] : 0.0f;
    }
}

__global__ void convert_to_f64(double* __restrict__ d, const float* __restrict__ s, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        d[q] = (double)s[q];
}

int ensure_stage(SeidartSolver& s, size_t n) {
    if (s.stage && s.stage_n >= n) return SEIDART_OK;
    if (s.stage) cudaFree(s.stage);
    s.stage = nullptr;
    s.stage_n = 0;
    if (cudaMalloc((void**)&s.stage, n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return SEIDART_ERR_NOMEM;
    }
    s.stage_n = n;
    return SEIDART_OK;
}

// FP32 transfers of large arrays go through a pinned double buffer: on the
// way in, host threads round chunk k of the caller's FP64 array (in the
// derived form of `mode`, the same FP64 operations as convert_to_f32) into
// one half while chunk k-1 is copied from the other; on the way out, chunk
// k is widened into the caller's array while chunk k+1 is copied.  Half the
// bytes of FP64 cross the link, and no staging kernel runs.
constexpr size_t kPinChunk = size_t(1) << 23;  // floats per chunk (32 MiB)

int ensure_pin(SeidartSolver& s) {
    if (s.pin) return SEIDART_OK;
    if (cudaMallocHost((void**)&s.pin, 2 * kPinChunk * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        s.pin = nullptr;
        return SEIDART_ERR_NOMEM;
    }
    for (int b = 0; b < 2; ++b) CUDA_TRY(cudaEventCreateWithFlags(&s.pin_ev[b], cudaEventDisableTiming));
    return SEIDART_OK;
}

using seidart_host::host_parallel;  // body(lo, hi) over [0, m) on the host thread pool

void widen(double* dst, const float* src, size_t m) {
    host_parallel(m, [&](size_t lo, size_t hi) {
        for (size_t q = lo; q < hi; ++q) dst[q] = (double)src[q];
    });
}

void narrow(float* dst, const double* src, size_t m, int mode, double dt) {
    host_parallel(m, [&](size_t lo, size_t hi) {
        for (size_t q = lo; q < hi; ++q) {
            double x = src[q];
            if (mode == 1) x = 1.0 / (1.0 + x * dt);
            else if (mode == 2) x = 1.0 / x;
            dst[q] = (float)x;
        }
    });
}

int upload_f32_pinned(SeidartSolver& s, float* d, const double* h, size_t n, int mode) {
    cudaStream_t st = s.stream;
    if (const int rc = ensure_pin(s)) return rc;
    const size_t nch = (n + kPinChunk - 1) / kPinChunk;
    for (size_t k = 0; k < nch; ++k) {
        const int b = (int)(k & 1);
        if (k >= 2) CUDA_TRY(cudaEventSynchronize(s.pin_ev[b]));  // the copy that last read this half
        const size_t o = k * kPinChunk, m = std::min(kPinChunk, n - o);
        narrow(s.pin + b * kPinChunk, h + o, m, mode, s.src.dt);
        CUDA_TRY(cudaMemcpyAsync(d + o, s.pin + b * kPinChunk, m * sizeof(float), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaEventRecord(s.pin_ev[b], st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return SEIDART_OK;
}

int download_f32_pinned(SeidartSolver& s, double* h, const float* d, size_t n) {
    cudaStream_t st = s.stream;
    if (const int rc = ensure_pin(s)) return rc;
    const size_t nch = (n + kPinChunk - 1) / kPinChunk;
    auto issue = [&](size_t k) -> cudaError_t {
        const size_t o = k * kPinChunk, m = std::min(kPinChunk, n - o);
        cudaError_t e = cudaMemcpyAsync(s.pin + (k & 1) * kPinChunk, d + o, m * sizeof(float), cudaMemcpyDeviceToHost, st);
        return e == cudaSuccess ? cudaEventRecord(s.pin_ev[k & 1], st) : e;
    };
    if (nch > 0) CUDA_TRY(issue(0));
    for (size_t k = 0; k < nch; ++k) {
        if (k + 1 < nch) CUDA_TRY(issue(k + 1));
        CUDA_TRY(cudaEventSynchronize(s.pin_ev[k & 1]));
        const size_t o = k * kPinChunk, m = std::min(kPinChunk, n - o);
        widen(h + o, s.pin + (k & 1) * kPinChunk, m);
    }
    return SEIDART_OK;
}

// true when p is device memory (a model grid produced on the device, e.g. by
// the device material pre-pass); such arrays are copied or converted device
// to device
bool is_device_ptr(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice;
}

template <typename T>
int upload(SeidartSolver& s, void* d, const double* h, size_t n, int mode = 0) {
    cudaStream_t st = s.stream;
    if (h && is_device_ptr(h)) {
        if (sizeof(T) == sizeof(double)) {
            CUDA_TRY(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            if (mode != 0 && n > 0) derive_f64<<<4 * 152, 256, 0, st>>>((double*)d, n, mode, s.src.dt);
        } else if (n > 0) {
            convert_to_f32<<<4 * 152, 256, 0, st>>>((float*)d, h, n, mode, s.src.dt);
        }
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(st));
        return SEIDART_OK;
    }
    if (sizeof(T) == sizeof(double)) {
        CUDA_TRY(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, st));
        if (mode != 0 && n > 0) {
            derive_f64<<<4 * 152, 256, 0, st>>>((double*)d, n, mode, s.src.dt);
            CUDA_TRY(cudaGetLastError());
        }
        CUDA_TRY(cudaStreamSynchronize(st));
        return SEIDART_OK;
    }
    if (n >= kPinChunk / 4) {  // large arrays: pinned FP32 path (falls through if no pinned memory)
        const int rc = upload_f32_pinned(s, (float*)d, h, n, mode);
        if (rc != SEIDART_ERR_NOMEM) return rc;
    }
    const size_t chunk = std::max<size_t>(s.ncell, 1 << 20);
    if (ensure_stage(s, std::min(n, chunk)) != SEIDART_OK) return set_err(SEIDART_ERR_NOMEM, "staging buffer");
    for (size_t o = 0; o < n; o += s.stage_n) {
        const size_t m = std::min(s.stage_n, n - o);
        CUDA_TRY(cudaMemcpyAsync(s.stage, h + o, m * sizeof(double), cudaMemcpyHostToDevice, st));
        convert_to_f32<<<4 * 152, 256, 0, st>>>((float*)d + o, s.stage, m, mode, s.src.dt);
        CUDA_TRY(cudaGetLastError());
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return SEIDART_OK;
}
template <typename T>
int download(SeidartSolver& s, double* h, const void* d, size_t n) {
    cudaStream_t st = s.stream;
    if (sizeof(T) == sizeof(double)) {
        CUDA_TRY(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return SEIDART_OK;
    }
    if (n >= kPinChunk / 4) {  // large arrays: pinned FP32 path (falls through if no pinned memory)
        const int rc = download_f32_pinned(s, h, (const float*)d, n);
        if (rc != SEIDART_ERR_NOMEM) return rc;
    }
    const size_t chunk = std::max<size_t>(s.ncell, 1 << 20);
    if (ensure_stage(s, std::min(n, chunk)) != SEIDART_OK) return set_err(SEIDART_ERR_NOMEM, "staging buffer");
    for (size_t o = 0; o < n; o += s.stage_n) {
        const size_t m = std::min(s.stage_n, n - o);
        convert_to_f64<<<4 * 152, 256, 0, st>>>(s.stage, (const float*)d + o, m);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(h + o, s.stage, m * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return SEIDART_OK;
}

// Interior box: the largest box found inside [cpml, n-cpml) per axis whose
// cells all have inert CPML coefficients (acoef = acoef_half = 0,
// kappa = kappa_half = 1, finite b).  Starting from the nominal box, faces
// that still hold active cells (e.g. the half-grid profile reaching one cell
// further on the high side) are peeled off a few times; the result is then
// verified cell by cell.  If verification fails the box is empty and the
// CPML arithmetic runs on every cell, as in the reference.
BoxH interior_box(const SeidartSolver& s, const double* const* model) {
    const int cs = cpml_slot(s.family);
    const double *kap = model[cs], *kaph = model[cs + 1], *ac = model[cs + 2], *ach = model[cs + 3],
                 *bc = model[cs + 4], *bch = model[cs + 5];
    const int nx = s.dom.nx, nz = s.dom.nz, c = s.dom.cpml;
    const bool is3 = s.family == SEIDART_SEISMIC3 || s.family == SEIDART_ELECTROMAG3;
    const int ny = is3 ? s.dom.ny : 1;
    BoxH b{c, nx - c, is3 ? c : 0, is3 ? ny - c : 1, c, nz - c};
    const BoxH empty{0, 0, 0, 0, 0, 0};
    auto active = [&](int i, int j, int k) {
        const size_t q = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
        return ac[q] != 0.0 || ach[q] != 0.0 || kap[q] != 1.0 || kaph[q] != 1.0 || !isfinite(bc[q]) ||
               !isfinite(bch[q]);
    };
    auto nonempty = [&]() { return b.i0 < b.i1 && b.j0 < b.j1 && b.k0 < b.k1; };
    // face test on plane `axis` = idx of the current box
    auto face = [&](int axis, int idx) {
        const int lo[3] = {b.i0, b.j0, b.k0}, hi[3] = {b.i1, b.j1, b.k1};
        int l[3] = {lo[0], lo[1], lo[2]}, h[3] = {hi[0], hi[1], hi[2]};
        l[axis] = idx; h[axis] = idx + 1;
        for (int k = l[2]; k < h[2]; ++k)
            for (int j = l[1]; j < h[1]; ++j)
                for (int i = l[0]; i < h[0]; ++i)
                    if (active(i, j, k)) return true;
        return false;
    };
    for (int it = 0; it < 4 && nonempty(); ++it) {
        bool changed = false;
        if (face(0, b.i0)) { ++b.i0; changed = true; }
        if (nonempty() && face(0, b.i1 - 1)) { --b.i1; changed = true; }
        if (is3 && nonempty() && face(1, b.j0)) { ++b.j0; changed = true; }
        if (is3 && nonempty() && face(1, b.j1 - 1)) { --b.j1; changed = true; }
        if (nonempty() && face(2, b.k0)) { ++b.k0; changed = true; }
        if (nonempty() && face(2, b.k1 - 1)) { --b.k1; changed = true; }
        if (!changed) break;
    }
    if (!nonempty()) return empty;
    // cell-by-cell verification, z planes shared out over host threads (on
    // the 352^3 grid one thread takes 84 ms)
    seidart_host::HostPool& pool = seidart_host::HostPool::get();
    const int nth = (int)std::min<long>(pool.size(), (long)(b.k1 - b.k0));
    std::atomic<bool> bad{false};
    pool.run(nth, [&](int w) {
        for (int k = b.k0 + w; k < b.k1 && !bad.load(std::memory_order_relaxed); k += nth)
            for (int j = b.j0; j < b.j1; ++j)
                for (int i = b.i0; i < b.i1; ++i)
                    if (active(i, j, k)) { bad = true; return; }
    });
    return bad ? empty : b;
}

// Model set-up per family; `T` is the field precision.
template <typename T>
int setup_model(SeidartSolver& s, const double* const* model, const double* const* srcfn,
                const double** dev_src, std::vector<std::vector<double>>& derived) {
    const size_t N = s.ncell;
    // reciprocal forms of the fast arithmetic (FP32 and fast FP64 solvers)
    const bool recip = sizeof(T) == sizeof(float) || s.precision == SEIDART_FP64_FAST;
    const double dt = s.src.dt;
    auto arr = [&](const double* h) -> const T* {
        T* d = (T*)s.carve(N * sizeof(T));
        if (d && upload<T>(s, d, h, N) != SEIDART_OK) return nullptr;
        return d;
    };
    // arrays of a derived form, converted on the device (mode of convert_to_f32 / derive_f64)
    auto arr_mode = [&](const double* h, int mode) -> const T* {
        T* d = (T*)s.carve(N * sizeof(T));
        if (d && upload<T>(s, d, h, N, mode) != SEIDART_OK) return nullptr;
        return d;
    };
    // while measuring (no arena yet) only sizes matter: skip the arithmetic
    static const double dummy = 0.0;
    auto derive = [&](auto fn) -> const double* {
        if (!s.arena) return &dummy;
        derived.emplace_back(N);
        std::vector<double>& v = derived.back();
        for (size_t q = 0; q < N; ++q) v[q] = fn(q);
        return v.data();
    };
    // fast arithmetic: gamma -> 1/(1+gamma dt), kappa -> 1/kappa (same memory traffic)
    auto gam = [&](const double* g) { return recip ? arr_mode(g, 1) : arr(g); };
    auto kap = [&](const double* k) { return recip ? arr_mode(k, 2) : arr(k); };
    (void)dt;
    const int cs = cpml_slot(s.family);
    const T* cp[6];
    cp[0] = kap(model[cs]);
    cp[1] = kap(model[cs + 1]);
    for (int q = 2; q < 6; ++q) cp[q] = arr(model[cs + q]);

    switch (s.family) {
    case SEIDART_SEISMIC2: {
        S2Args<T> a{};
        for (int q = 0; q < 7; ++q) a.m[q] = arr(model[q]);
        for (int q = 7; q < 10; ++q) a.m[q] = gam(model[q]);
        for (int q = 0; q < 6; ++q) a.m[10 + q] = cp[q];
        for (int q = 0; q < 5; ++q) a.src[q] = dev_src[q];
        if constexpr (sizeof(T) == 8) s.s2d = a; else s.s2f = a;
        break;
    }
    case SEIDART_ELECTROMAG2: {
        // cpmlfdtd.f08:2519-2540
        const double *e11 = model[E2_E11], *e13 = model[E2_E13], *e33 = model[E2_E33], *s11 = model[E2_S11],
                     *s13 = model[E2_S13], *s33 = model[E2_S33];
        std::vector<double> det(s.arena ? N : 0);
        for (size_t q = 0; q < det.size(); ++q) {
            const double a11 = e11[q] * kEps0, a13 = e13[q] * kEps0, a33 = e33[q] * kEps0;
            double d = a11 * a33 - a13 * a13;
            if (d <= 1.0e-18 * kEps0 * kEps0) d = 1.0e-18 * kEps0 * kEps0;
            det[q] = d;
        }
        auto A = [&](size_t q, int which) {
            const double a11 = e11[q] * kEps0, a13 = e13[q] * kEps0, a33 = e33[q] * kEps0, d = det[q];
            switch (which) {
            case 0: return a33 / d;
            case 1: return -a13 / d;
            case 2: return (a33 * s11[q] - a13 * s13[q]) / d;
            case 3: return (a33 * s13[q] - a13 * s33[q]) / d;
            case 4: return -a13 / d;
            case 5: return a11 / d;
            case 6: return (a11 * s13[q] - a13 * s11[q]) / d;
            case 7: return (a11 * s33[q] - a13 * s13[q]) / d;
            case 8: return a11;
            default: return a33;
            }
        };
        E2Args<T> a{};
        for (int w = 0; w < 10; ++w) a.c[w] = arr(derive([&](size_t q) { return A(q, w); }));
        for (int q = 0; q < 6; ++q) a.cpml[q] = cp[q];
        for (int q = 0; q < 2; ++q) a.src[q] = dev_src[q];
        if constexpr (sizeof(T) == 8) s.e2d = a; else s.e2f = a;
        break;
    }
    case SEIDART_SEISMIC25: {
        S25Args<T> a{};
        for (int q = 0; q < 21; ++q) a.C[q] = arr(model[q]);
        for (int q = 0; q < 6; ++q) a.g[q] = gam(model[SEIDART_GX3 + q]);
        for (int q = 0; q < 6; ++q) a.cpml[q] = cp[q];
        // density averaging, cpmlfdtd.f08:889-898 (fast arithmetic: stored as 1/rho)
        const double* rho = model[SEIDART_RHO3];
        const int dirs[9] = {0, -1, 2, 1, -1, 2, 1, -1, 3};  // -1: plain rho
        for (int q = 0; q < 9; ++q) {
            if (!s.arena) { a.rho9[q] = arr(rho); continue; }
            derived.emplace_back(rho, rho + N);
            if (dirs[q] >= 0) averaging2d(derived.back().data(), s.dom.nx, s.dom.nz, s.density, dirs[q]);
            if (recip) for (double& v : derived.back()) v = 1.0 / v;
            a.rho9[q] = arr(derived.back().data());
        }
        a.rho = recip ? arr_mode(rho, 2) : arr(rho);
        for (int q = 0; q < 9; ++q) a.src[q] = dev_src[q];
        if constexpr (sizeof(T) == 8) s.s25d = a; else s.s25f = a;
        break;
    }
    case SEIDART_ELECTROMAG25: {
        // cpmlfdtd.f08:3046-3067
        std::vector<double> det(s.arena ? N : 0);
        const double* E[6];
        for (int q = 0; q < 6; ++q) E[q] = model[E25_E11 + q];
        auto ee = [&](int w, size_t q) { return E[w][q] * kEps0; };  // 0 e11 1 e12 2 e13 3 e22 4 e23 5 e33
        for (size_t q = 0; q < det.size(); ++q) {
            const double a11 = ee(0, q), a12 = ee(1, q), a13 = ee(2, q), a22 = ee(3, q), a23 = ee(4, q), a33 = ee(5, q);
            det[q] = a11 * (a22 * a33 - a23 * a23) - a12 * (a12 * a33 - a23 * a13) + a13 * (a12 * a23 - a22 * a13);
        }
        auto inv = [&](size_t q, int w) {
            const double a11 = ee(0, q), a12 = ee(1, q), a13 = ee(2, q), a22 = ee(3, q), a23 = ee(4, q), a33 = ee(5, q);
            const double d = det[q];
            const double aEx = (a22 * a33 - a23 * a23) / d, bEx = -((a12 * a33 - a23 * a13) / d),
                         cEx = (a12 * a23 - a22 * a13) / d, bEy = (a11 * a33 - a13 * a13) / d,
                         cEy = -((a11 * a23 - a12 * a13) / d), cEz = (a11 * a22 - a12 * a12) / d;
            const double v[9] = {aEx, bEx, cEx, bEx, bEy, cEy, cEx, cEy, cEz};
            return v[w];
        };
        E25Args<T> a{};
        for (int w = 0; w < 9; ++w) a.inv[w] = arr(derive([&](size_t q) { return inv(q, w); }));
        for (int w = 0; w < 6; ++w) a.sig[w] = arr(model[E25_S11 + w]);
        const int ed[3] = {0, 3, 5};
        for (int w = 0; w < 3; ++w) a.eabs[w] = arr(derive([&](size_t q) { return ee(ed[w], q); }));
        for (int q = 0; q < 6; ++q) a.cpml[q] = cp[q];
        for (int q = 0; q < 3; ++q) a.src[q] = dev_src[q];
        if constexpr (sizeof(T) == 8) s.e25d = a; else s.e25f = a;
        break;
    }
    case SEIDART_ELECTROMAG3: {
        // cpmlfdtd.f08:3643-3666 (the same inverse as electromag25, no clamp)
        std::vector<double> det(s.arena ? N : 0);
        const double* E[6];
        for (int q = 0; q < 6; ++q) E[q] = model[E3_E11 + q];
        auto ee = [&](int w, size_t q) { return E[w][q] * kEps0; };  // 0 e11 1 e12 2 e13 3 e22 4 e23 5 e33
        for (size_t q = 0; q < det.size(); ++q) {
            const double a11 = ee(0, q), a12 = ee(1, q), a13 = ee(2, q), a22 = ee(3, q), a23 = ee(4, q), a33 = ee(5, q);
            det[q] = a11 * (a22 * a33 - a23 * a23) - a12 * (a12 * a33 - a23 * a13) + a13 * (a12 * a23 - a22 * a13);
        }
        auto inv = [&](size_t q, int w) {
            const double a11 = ee(0, q), a12 = ee(1, q), a13 = ee(2, q), a22 = ee(3, q), a23 = ee(4, q), a33 = ee(5, q);
            const double d = det[q];
            const double aEx = (a22 * a33 - a23 * a23) / d, bEx = -((a12 * a33 - a23 * a13) / d),
                         cEx = (a12 * a23 - a22 * a13) / d, bEy = (a11 * a33 - a13 * a13) / d,
                         cEy = -((a11 * a23 - a12 * a13) / d), cEz = (a11 * a22 - a12 * a12) / d;
            const double v[9] = {aEx, bEx, cEx, bEx, bEy, cEy, cEx, cEy, cEz};
            return v[w];
        };
        E3Args<T> a{};
        for (int w = 0; w < 9; ++w) a.inv[w] = arr(derive([&](size_t q) { return inv(q, w); }));
        for (int w = 0; w < 6; ++w) a.sig[w] = arr(model[E3_S11 + w]);
        const int ed[3] = {0, 3, 5};
        for (int w = 0; w < 3; ++w) a.eabs[w] = arr(derive([&](size_t q) { return ee(ed[w], q); }));
        for (int q = 0; q < 6; ++q) a.cpml[q] = cp[q];
        for (int q = 0; q < 3; ++q) a.src[q] = dev_src[q];
        if constexpr (sizeof(T) == 8) s.e3d = a; else s.e3f = a;
        break;
    }
    case SEIDART_SEISMIC3: {
        S3Args<T> a{};
        for (int q = 0; q < 21; ++q) a.C[q] = arr(model[q]);
        a.rho = arr(model[SEIDART_RHO3]);
        for (int q = 0; q < 6; ++q) a.g[q] = gam(model[SEIDART_GX3 + q]);
        for (int q = 0; q < 6; ++q) a.cpml[q] = cp[q];
        for (int q = 0; q < 9; ++q) a.src[q] = dev_src[q];
        if constexpr (sizeof(T) == 8) s.s3d = a; else s.s3f = a;
        break;
    }
    }
    (void)srcfn;
    return SEIDART_OK;
}

// Fill the per-family scalar fields and state pointers of the arg blocks.
template <typename T, typename A>
void fill_common2(SeidartSolver& s, A& a) {
    a.nx = s.dom.nx; a.nz = s.dom.nz;
    a.dt = (T)s.src.dt;
    a.box = s.box;
    a.traces = (T*)s.traces;
    a.norms = s.norms;
    for (size_t q = 0; q < s.fields.size(); ++q) a.f[q] = (T*)s.fields[q];
    for (size_t q = 0; q < s.mem.size(); ++q) a.mem[q] = (T*)s.mem[q];
}

template <typename T>
void finish_args(SeidartSolver& s) {
    const int is = s.src.xind + s.dom.cpml - 1, js = s.src.yind + s.dom.cpml - 1, ks = s.src.zind + s.dom.cpml - 1;
    const bool f32 = sizeof(T) == sizeof(float);
    const bool recip = f32 || s.precision == SEIDART_FP64_FAST;
    switch (s.family) {
    case SEIDART_SEISMIC2: {
        S2Args<T>& a = *(S2Args<T>*)(f32 ? (void*)&s.s2f : (void*)&s.s2d);
        fill_common2<T>(s, a);
        a.dx = (T)s.dom.dx; a.dz = (T)s.dom.dz; a.density_code = s.density;
        a.isrc = is; a.jsrc = ks; a.stress_src = s.stress_src;
        break;
    }
    case SEIDART_ELECTROMAG2: {
        E2Args<T>& a = *(E2Args<T>*)(f32 ? (void*)&s.e2f : (void*)&s.e2d);
        fill_common2<T>(s, a);
        // the fast builds multiply by 1/dx, 1/dz
        a.dx = recip ? (T)(1.0 / s.dom.dx) : (T)s.dom.dx;
        a.dz = recip ? (T)(1.0 / s.dom.dz) : (T)s.dom.dz;
        a.dbHy = (T)(s.src.dt / kMu0);
        a.isrc = is; a.jsrc = ks;
        break;
    }
    case SEIDART_SEISMIC25: {
        S25Args<T>& a = *(S25Args<T>*)(f32 ? (void*)&s.s25f : (void*)&s.s25d);
        fill_common2<T>(s, a);
        a.dx = (T)s.dom.dx; a.dz = (T)s.dom.dz; a.ky = (T)s.src.ky;
        a.isrc = is; a.ksrc = ks; a.stress_src = s.stress_src;
        break;
    }
    case SEIDART_ELECTROMAG25: {
        E25Args<T>& a = *(E25Args<T>*)(f32 ? (void*)&s.e25f : (void*)&s.e25d);
        fill_common2<T>(s, a);
        a.dx = (T)s.dom.dx; a.dz = (T)s.dom.dz; a.ky = (T)s.src.ky;
        a.dtmu = (T)(s.src.dt / kMu0);
        a.isrc = is; a.ksrc = ks;
        break;
    }
    case SEIDART_ELECTROMAG3: {
        E3Args<T>& a = *(E3Args<T>*)(f32 ? (void*)&s.e3f : (void*)&s.e3d);
        fill_common2<T>(s, a);
        a.ny = s.dom.ny;
        // the fast builds multiply by 1/dx, 1/dy, 1/dz
        a.dx = recip ? (T)(1.0 / s.dom.dx) : (T)s.dom.dx;
        a.dy = recip ? (T)(1.0 / s.dom.dy) : (T)s.dom.dy;
        a.dz = recip ? (T)(1.0 / s.dom.dz) : (T)s.dom.dz;
        a.dbH = (T)(s.src.dt / kMu0);
        a.isrc = is; a.jsrc = js; a.ksrc = ks;
        break;
    }
    case SEIDART_SEISMIC3: {
        S3Args<T>& a = *(S3Args<T>*)(f32 ? (void*)&s.s3f : (void*)&s.s3d);
        fill_common2<T>(s, a);
        a.ny = s.dom.ny;
        a.dx = (T)s.dom.dx; a.dy = (T)s.dom.dy; a.dz = (T)s.dom.dz; a.density_code = s.density;
        a.isrc = is; a.jsrc = js; a.ksrc = ks; a.stress_src = s.stress_src;
        a.nt = s.src.time_steps;
        a.norms_part = s.norms_part;
        a.err = s.err_dev;
        a.wait_limit = 1 << 20;
        a.wait_probe = 0;
        a.wave_ctl = nullptr;  // set once the fused step is prepared
        a.wave_n = 0;
        break;
    }
    }
}

const PwDev& solver_pw(const SeidartSolver& s) {
    const bool f = s.precision == SEIDART_FP32;
    switch (s.family) {
    case SEIDART_SEISMIC2: return f ? s.s2f.pw : s.s2d.pw;
    case SEIDART_SEISMIC25: return f ? s.s25f.pw : s.s25d.pw;
    case SEIDART_SEISMIC3: return f ? s.s3f.pw : s.s3d.pw;
    case SEIDART_ELECTROMAG2: return f ? s.e2f.pw : s.e2d.pw;
    case SEIDART_ELECTROMAG3: return f ? s.e3f.pw : s.e3d.pw;
    default: return f ? s.e25f.pw : s.e25d.pw;
    }
}

// kernels per step: update pair + epilogue, the stress-source kernel, and a
// plane wave's face launches plus its norm launch
int launches_per_step(const SeidartSolver& s) {
    const PwDev& pw = solver_pw(s);
    // the fused 3D step replaces the two half-step kernels by one
    const bool wave = s.family == SEIDART_SEISMIC3 && s.precision == SEIDART_FP32 && !pw.on && s.s3f.wave_ctl &&
                      s.s3f.staged;
    return (wave ? 2 : 3) + (s.stress_src ? 1 : 0) + (pw.on && pw.nface > 0 ? pw.nface + 1 : 0);
}

void launch_one_step(SeidartSolver& s, cudaStream_t st, const LaunchHook* h = nullptr) {
    StepInfo si{s.step_dev, s.nrec, s.rec_dev};
    const bool f32 = s.precision == SEIDART_FP32, fx = s.precision == SEIDART_FP64_FAST;
    // FP64 solvers: the exact build, or the fast-arithmetic FP64 build
#define SD_F64(fam, args) (fx ? launch_##fam##_f64x(args, si, st, h) : launch_##fam##_f64(args, si, st, h))
    switch (s.family) {
    case SEIDART_SEISMIC2: f32 ? launch_seismic2_f32(s.s2f, si, st, h) : SD_F64(seismic2, s.s2d); break;
    case SEIDART_ELECTROMAG2: f32 ? launch_electromag2_f32(s.e2f, si, st, h) : SD_F64(electromag2, s.e2d); break;
    case SEIDART_SEISMIC25: f32 ? launch_seismic25_f32(s.s25f, si, st, h) : SD_F64(seismic25, s.s25d); break;
    case SEIDART_ELECTROMAG25: f32 ? launch_electromag25_f32(s.e25f, si, st, h) : SD_F64(electromag25, s.e25d); break;
    case SEIDART_ELECTROMAG3: f32 ? launch_electromag3_f32(s.e3f, si, st, h) : SD_F64(electromag3, s.e3d); break;
    case SEIDART_SEISMIC3:
        if (!f32) SD_F64(seismic3, s.s3d);
        else launch_seismic3_fast(s.s3f, si, st, h, s.s3_tma ? &s.s3_maps : nullptr, s.s3_stress_kind,
                                  s.s3_velocity_kind);
        break;
    }
#undef SD_F64
}

// Event recorder for seidart_solver_profile: one event after every kernel.
struct EventLog {
    cudaStream_t st;
    std::vector<cudaEvent_t> ev;
    std::vector<int> kid;
    std::vector<std::string> names;
    size_t next = 0;
    bool failed = false;
    static void on_launch(void* ctx, int k, const char* name) {
        EventLog* L = (EventLog*)ctx;
        if (L->next >= L->ev.size()) { L->failed = true; return; }
        if (cudaEventRecord(L->ev[L->next], L->st) != cudaSuccess) L->failed = true;
        L->kid[L->next] = k;
        if ((int)L->names.size() <= k) L->names.resize(k + 1);
        L->names[k] = name;
        ++L->next;
    }
};

int graph_for(SeidartSolver& s, int len, cudaGraphExec_t* out) {
    for (int q = 0; q < 2; ++q)
        if (s.graph_exec[q] && s.graph_len[q] == len) { *out = s.graph_exec[q]; return SEIDART_OK; }
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
    for (int t = 0; t < len; ++t) launch_one_step(s, s.stream);
    CUDA_TRY(cudaStreamEndCapture(s.stream, &g));
    cudaGraphExec_t ex = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(SEIDART_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    // keep at most two cached lengths (the chunk and a tail)
    int slot = s.graph_exec[0] == nullptr ? 0 : 1;
    if (s.graph_exec[slot]) cudaGraphExecDestroy(s.graph_exec[slot]);
    s.graph_exec[slot] = ex;
    s.graph_len[slot] = len;
    *out = ex;
    return SEIDART_OK;
}

}  // namespace

// kernels one step launches: half-step kernels, optional stress source, epilogue
int seidart_step_launches(int family, int stress_src) {
    (void)family;
    return 3 + (stress_src ? 1 : 0);
}

extern "C" {

const char* seidart_last_error(void) { return g_err.c_str(); }
// error text for entry points defined in other files (read back through
// seidart_last_error); not part of the ABI
int seidart_internal_set_error(int code, const char* msg) { return set_err(code, "%s", msg); }

int seidart_layout(int family, int* nmodel, int* nsrc, int* nfield, int* nmem, int* is_complex, int* nrec_comp) {
    Layout L;
    if (!layout_of(family, &L)) return set_err(SEIDART_ERR_ARG, "unknown solver family %d", family);
    if (nmodel) *nmodel = L.nmodel;
    if (nsrc) *nsrc = L.nsrc;
    if (nfield) *nfield = L.nfield;
    if (nmem) *nmem = L.nmem;
    if (is_complex) *is_complex = L.cplx;
    if (nrec_comp) *nrec_comp = L.ncomp;
    return SEIDART_OK;
}

namespace {
// Set-up stage times on stderr when SEIDART_TRACE_SETUP=1; each mark first
// waits for the solver's stream, so a stage's device work counts in it.
struct SetupTrace {
    bool on;
    std::chrono::steady_clock::time_point last;
    SetupTrace() {
        const char* t = getenv("SEIDART_TRACE_SETUP");
        on = t && *t == '1';
        last = std::chrono::steady_clock::now();
    }
    void mark(const char* stage, cudaStream_t st = nullptr) {
        if (!on) return;
        if (st) cudaStreamSynchronize(st);
        const auto t = std::chrono::steady_clock::now();
        fprintf(stderr, "seidart set-up: %-24s %9.2f ms\n", stage,
                std::chrono::duration<double, std::milli>(t - last).count());
        last = t;
    }
};
}  // namespace

int seidart_solver_create(SeidartSolver** out, int family, int precision, const SeidartDomain* dom,
                          const SeidartSource* src, int density_code, const double* const* model,
                          const double* const* srcfn, int nrec, const int* rec_cells) {
    if (!out || !dom || !src || !model) return set_err(SEIDART_ERR_ARG, "NULL argument");
    *out = nullptr;
    SetupTrace trace;
    seidart_trace::Range nvtx("seidart_solver_create");
    Layout L;
    if (!layout_of(family, &L)) return set_err(SEIDART_ERR_ARG, "unknown solver family %d", family);
    if (precision != SEIDART_FP64 && precision != SEIDART_FP32 && precision != SEIDART_FP64_FAST)
        return set_err(SEIDART_ERR_ARG, "precision must be SEIDART_FP64, SEIDART_FP32 or SEIDART_FP64_FAST");
    if (density_code < 1 || density_code > 4)
        return set_err(SEIDART_ERR_ARG, "density_code %d: must be 1 harmonic, 2 geometric, 3 arithmetic, 4 none",
                       density_code);
    const bool is3 = family == SEIDART_SEISMIC3 || family == SEIDART_ELECTROMAG3;
    const int nx = dom->nx, nz = dom->nz, ny = is3 ? dom->ny : 1;
    if (nx < 6 || nz < 6 || (is3 && ny < 6)) return set_err(SEIDART_ERR_ARG, "grid too small (need >= 6 cells per axis)");
    if (src->time_steps < 1) return set_err(SEIDART_ERR_ARG, "time_steps must be >= 1");
    if (!(src->dt > 0)) return set_err(SEIDART_ERR_ARG, "dt must be > 0");
    if (!(dom->dx > 0) || !(dom->dz > 0) || (is3 && !(dom->dy > 0))) return set_err(SEIDART_ERR_ARG, "grid spacing must be > 0");
    // the source cell and its staggered neighbours (+1) must lie inside the grid
    const int is = src->xind + dom->cpml - 1, js = src->yind + dom->cpml - 1, ks = src->zind + dom->cpml - 1;
    if (is < 0 || is + 1 >= nx || ks < 0 || ks + 1 >= nz || (is3 && (js < 0 || js + 1 >= ny)))
        return set_err(SEIDART_ERR_ARG, "source index (%d,%d,%d)+cpml outside the padded grid", src->xind, src->yind, src->zind);
    for (int q = 0; q < L.nmodel; ++q)
        if (!model[q]) return set_err(SEIDART_ERR_ARG, "model array %d is NULL", q);
    // device-resident model grids: the stiffness, density and attenuation
    // slots of seismic2 and seismic3 (their set-up only copies or converts
    // them); every other array is read on the host during set-up
    {
        const bool dev_ok = family == SEIDART_SEISMIC2 || family == SEIDART_SEISMIC3;
        const int first_cpml = cpml_slot(family);
        for (int q = 0; q < L.nmodel; ++q)
            if (is_device_ptr(model[q]) && (!dev_ok || q >= first_cpml))
                return set_err(SEIDART_ERR_ARG,
                               "model array %d is device memory: only the stiffness, density and attenuation grids "
                               "of seismic2 and seismic3 may be", q);
    }
    const size_t N = (size_t)nx * ny * nz;
    for (int r = 0; r < nrec; ++r)
        if (!rec_cells || rec_cells[r] < 0 || (size_t)rec_cells[r] >= N)
            return set_err(SEIDART_ERR_ARG, "receiver %d cell index out of range", r);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_err(SEIDART_ERR_UNSUPPORTED, "no CUDA device: the solvers run only on the GPU");

    SeidartSolver* s = new SeidartSolver();
    s->family = family; s->precision = precision; s->density = density_code;
    s->dom = *dom; s->src = *src; s->L = L;
    if (!is3) s->dom.ny = 1;
    s->ncell = N;
    s->esize = precision == SEIDART_FP32 ? 4 : 8;
    s->nrec = nrec;
    s->nnorm = family == SEIDART_SEISMIC3 ? 2 : 1;  // seismic3 also tracks the stress norm
    {
        auto kind = [](const char* e, int dflt) {
            const char* v = getenv(e);
            if (!v) return dflt;
            return strcmp(v, "zmarch") == 0 ? (int)S3K_ZMARCH
                   : strcmp(v, "tma") == 0  ? (int)S3K_TMA
                   : strcmp(v, "bulk") == 0 ? (int)S3K_BULK
                                            : (int)S3K_CELL;
        };
        s->s3_stress_kind = kind("SEIDART_S3_STRESS", s->s3_stress_kind);
        s->s3_velocity_kind = kind("SEIDART_S3_VELOCITY", s->s3_velocity_kind);
    }
    trace.mark("checks");
    s->box = interior_box(*s, model);
    trace.mark("interior box");
    for (int q = 0; q < L.nsrc; ++q) {
        // stress-source series are every slot after the force components
        const int first_stress = (family == SEIDART_SEISMIC2) ? S2_SRCXX : ((family == SEIDART_SEISMIC3 || family == SEIDART_SEISMIC25) ? S3_SRCXX : 1 << 20);
        if (q >= first_stress && srcfn && srcfn[q])
            for (int t = 0; t < src->time_steps; ++t)
                if (srcfn[q][t] != 0.0) { s->stress_src = 1; break; }
    }
    const int cf = L.cplx ? 2 : 1;
    // two passes: measure, then allocate and carve for real
    std::vector<std::vector<double>> derived;
    for (int pass = 0; pass < 2; ++pass) {
        s->arena_used = 0;
        s->fields.assign(L.nfield, nullptr);
        s->mem.assign(L.nmem, nullptr);
        for (int q = 0; q < L.nfield; ++q) s->fields[q] = s->carve(N * cf * s->esize);
        for (int q = 0; q < L.nmem; ++q) s->mem[q] = s->carve(N * cf * s->esize);
        const double* dsrc[9] = {nullptr};
        std::vector<std::pair<double*, int>> src_up;
        for (int q = 0; q < L.nsrc; ++q) {
            if (srcfn && srcfn[q]) {
                dsrc[q] = (const double*)s->carve(sizeof(double) * src->time_steps);
                src_up.push_back({(double*)dsrc[q], q});
            }
        }
        s->step_dev = (int*)s->carve(sizeof(int));
        s->rec_dev = (int*)s->carve(sizeof(int) * (nrec > 0 ? nrec : 1));
        s->traces = s->carve((size_t)src->time_steps * L.ncomp * (nrec > 0 ? nrec : 1) * cf * s->esize);
        s->norms = (double*)s->carve(sizeof(double) * src->time_steps * s->nnorm);
        s->norms_part = (double*)s->carve(sizeof(double) * 2 * 64);
        s->err_dev = (int*)s->carve(sizeof(int));
        if (family == SEIDART_SEISMIC3 && precision == SEIDART_FP32) {
            s->wave_n = WAVE_DONE0 + s->dom.nz;
            s->wave_ctl = (int*)s->carve(sizeof(int) * s->wave_n);
        }
        if (pass == 0) {
            // model arrays: measured by running the set-up against a null arena
            derived.clear();
            int rc = precision == SEIDART_FP32 ? setup_model<float>(*s, model, srcfn, dsrc, derived)
                                               : setup_model<double>(*s, model, srcfn, dsrc, derived);
            if (rc != SEIDART_OK) { delete s; return rc; }
            s->arena_bytes = s->arena_used;
            cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) { delete s; return set_err(SEIDART_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
            s->own_stream = true;
            e = cudaMalloc((void**)&s->arena, s->arena_bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                cudaStreamDestroy(s->stream);
                const size_t mb = s->arena_bytes >> 20;
                delete s;
                return set_err(SEIDART_ERR_NOMEM, "device allocation of %zu MiB failed: %s", mb, cudaGetErrorString(e));
            }
            trace.mark("arena sizing + allocation");
        } else {
            int rc = SEIDART_OK;
            if (cudaMemsetAsync(s->arena, 0, s->arena_bytes, s->stream) != cudaSuccess) rc = SEIDART_ERR_CUDA;
            for (auto& p : src_up)
                if (rc == SEIDART_OK &&
                    cudaMemcpyAsync(p.first, srcfn[p.second], sizeof(double) * src->time_steps, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
                    rc = SEIDART_ERR_CUDA;
            if (rc == SEIDART_OK && nrec > 0 &&
                cudaMemcpyAsync(s->rec_dev, rec_cells, sizeof(int) * nrec, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
                rc = SEIDART_ERR_CUDA;
            const int one = 1;
            if (rc == SEIDART_OK && cudaMemcpyAsync(s->step_dev, &one, sizeof(int), cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
                rc = SEIDART_ERR_CUDA;
            if (rc == SEIDART_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = SEIDART_ERR_CUDA;
            trace.mark("zero state, sources");
            derived.clear();
            if (rc == SEIDART_OK)
                rc = precision == SEIDART_FP32 ? setup_model<float>(*s, model, srcfn, dsrc, derived)
                                               : setup_model<double>(*s, model, srcfn, dsrc, derived);
            if (rc != SEIDART_OK) {
                seidart_solver_destroy(s);
                return rc == SEIDART_ERR_CUDA ? set_err(rc, "device set-up failed: %s", cudaGetErrorString(cudaGetLastError())) : rc;
            }
        }
    }
    trace.mark("model upload", s->stream);
    if (precision == SEIDART_FP32) finish_args<float>(*s); else finish_args<double>(*s);
    if (family == SEIDART_SEISMIC3 && precision == SEIDART_FP32 && s->s3_stress_kind == S3K_TMA) {
        const char* t = getenv("SEIDART_S3_TMA");
        const int v = (t && *t >= '0' && *t <= '9') ? atoi(t) : s->s3_tma_variant;
        s->s3_tma = seismic3_tma_prepare(s->s3f, &s->s3_maps, v);
        if (!s->s3_tma) s->s3_stress_kind = S3K_CELL;  // grid does not meet the TMA rules
    }
    if (family == SEIDART_SEISMIC3 && precision == SEIDART_FP32) {
        // L2 prefetch distances in tiles (measured on 352^3: stress 2.98 -> 2.44 ms
        // at 8, velocity 1.49 -> 1.42 ms at 1216, about 2.5 z planes of tiles)
        const char* t = getenv("SEIDART_S3_PF");
        s->s3f.prefetch = (t && *t >= '0' && *t <= '9') ? atoi(t) : 8;
        t = getenv("SEIDART_S3_PFV");
        s->s3f.prefetch_v = (t && *t >= '0' && *t <= '9') ? atoi(t) : 1216;
        t = getenv("SEIDART_S3_VEL_MINB");
        s->s3f.velocity_minb = (t && *t >= '4' && *t <= '8') ? atoi(t) : 6;  // 6: 1.07 ms vs 1.19 ms at 4 (352^3)
        // the distances as offsets on the 32 x 8 x 1 tile grid of both kernels
        const int gx = (s->dom.nx + 31) / 32, gy = (s->dom.ny + 7) / 8;
        auto split = [&](int d, int* o) { o[0] = d % gx; o[1] = (d / gx) % gy; o[2] = d / (gx * gy); };
        split(s->s3f.prefetch, s->s3f.pf_d);
        split(s->s3f.prefetch_v, s->s3f.pfv_d);
        // cell-pair velocity kernel (two x-adjacent cells per thread, float2
        // loads) when every pair is 8-byte aligned; SEIDART_S3_VPAIR=0 turns it off
        t = getenv("SEIDART_S3_VPAIR");
        s->s3f.velocity_pair = (s->dom.nx % 2 == 0) && !(t && *t == '0');
        // the pair kernel holds two cells per thread: 4 CTAs per SM (352^3: 0.995 ms
        // against 1.14 ms at 5 and 1.015 ms for the one-cell kernel at 6)
        if (s->s3f.velocity_pair && !getenv("SEIDART_S3_VEL_MINB")) s->s3f.velocity_minb = 4;
        // warps make the lean test for their own two rows of the pair tile
        // (SEIDART_S3_VSUB=0: one test per 32 x 16 tile)
        t = getenv("SEIDART_S3_VSUB");
        s->s3f.velocity_sub = (t && *t == '0') ? 0 : 1;
        // the velocity kernel walks down from the planes the stress kernel
        // finished on (bit-identical; SEIDART_S3_VREV=0 turns it off).  The
        // stress kernel's read-once copies take an L2 evict-first policy only
        // on request (SEIDART_S3_L2HINT=1): it paid while the stress kernel
        // waited on its C-PML memories (2.200 -> 2.187 ms at 352^3) and costs
        // since their loads are batched (1.684 -> 1.758 ms)
        t = getenv("SEIDART_S3_L2HINT");
        s->s3f.l2_hint = (t && *t == '1') ? 1 : 0;
        t = getenv("SEIDART_S3_VREV");
        s->s3f.v_reverse = (t && *t == '0') ? 0 : 1;
        t = getenv("SEIDART_S3_PFP");
        const int pfp = (t && *t >= '0' && *t <= '9') ? atoi(t) : 608;
        const int gy2 = (s->dom.ny + 15) / 16;
        s->s3f.pfp_d[0] = pfp % gx; s->s3f.pfp_d[1] = (pfp / gx) % gy2; s->s3f.pfp_d[2] = pfp / (gx * gy2);
    }
    if (family == SEIDART_SEISMIC3 && precision == SEIDART_FP32 && s->s3_stress_kind == S3K_BULK) {
        const char* t = getenv("SEIDART_S3_BULK");
        s->s3f.bulk_variant = (t && *t >= '0' && *t <= '9') ? atoi(t) : 2;
        if (s->s3f.bulk_variant >= seismic3_bulk_variants()) s->s3f.bulk_variant = 0;
        // fully staged variant (TMA tiles for stresses and velocities) when the
        // grid allows it; SEIDART_S3_STAGED=0 keeps the bulk kernel
        const char* st = getenv("SEIDART_S3_STAGED");
        if (!(st && *st == '0') && seismic3_staged_prepare(s->s3f, &s->s3_staged)) s->s3f.staged = &s->s3_staged;
        trace.mark("staged kernel maps", s->stream);
        // material-indexed coefficients for the staged kernel when the model
        // allows them (SEIDART_S3_MATIDX=0 keeps the per-cell blocks)
        const char* mi = getenv("SEIDART_S3_MATIDX");
        if (s->s3f.staged && !(mi && *mi == '0') &&
            seismic3_material_index(s->s3f, s->dom.nx, s->dom.ny, s->dom.nz, &s->s3_mat_ids, &s->s3_mat_tab,
                                    &s->s3_nmat, s->stream) > 0) {
            s->s3f.mat_ids = s->s3_mat_ids;
            s->s3f.mat_tab = s->s3_mat_tab;
            s->s3f.mat_tab_bytes = (s->s3_nmat * 27 * (int)sizeof(float) + 15) / 16 * 16;
        }
        trace.mark("material index", s->stream);
        // the tile-packed per-cell coefficient block (27 words per cell, 4.7 GB
        // at 352^3) only where a kernel reads it: the per-cell layout, the bulk
        // kernel, and the fused step (its tiles read the block)
        const char* wv = getenv("SEIDART_S3_WAVE");
        const bool want_wave = wv && *wv == '1';
        if (!s->s3f.mat_ids || want_wave) {
            const size_t bytes = seismic3_bulk_bytes(s->dom.nx, s->dom.ny, s->dom.nz);
            if (cudaMalloc((void**)&s->s3_packed, bytes) != cudaSuccess) {
                cudaGetLastError();
                seidart_solver_destroy(s);
                return set_err(SEIDART_ERR_NOMEM, "cannot allocate %zu bytes for the packed 3D coefficients", bytes);
            }
            if (seismic3_bulk_pack(s->s3f, s->s3_packed, s->stream) != cudaSuccess ||
                cudaStreamSynchronize(s->stream) != cudaSuccess) {
                seidart_solver_destroy(s);
                return set_err(SEIDART_ERR_CUDA, "coefficient packing failed: %s",
                               cudaGetErrorString(cudaGetLastError()));
            }
            s->s3f.packed = s->s3_packed;
        }
        trace.mark("per-cell coefficient block", s->stream);
        // the six C-PML grids indexed the same way (a grid built from 1D
        // profiles holds a few dozen tuples; SEIDART_S3_CPMLIDX=0 keeps them)
        const char* ci = getenv("SEIDART_S3_CPMLIDX");
        if (s->s3f.staged && !(ci && *ci == '0') &&
            seismic3_cpml_index(s->s3f, s->dom.nx, s->dom.ny, s->dom.nz, &s->s3_cpml_ids, &s->s3_cpml_tab,
                                &s->s3_ncpml, s->stream) > 0) {
            s->s3f.cpml_ids = s->s3_cpml_ids;
            s->s3f.cpml_tab = s->s3_cpml_tab;
        }

        trace.mark("C-PML index", s->stream);
        // staged velocity kernel: bit-identical but measured slower at 352^3
        // (1.55 ms against 1.19 ms), so only on request
        const char* sv = getenv("SEIDART_S3_STAGED_V");
        if (s->s3f.staged && (sv && *sv == '1') && s->s3_velocity_kind == S3K_CELL &&
            seismic3_staged_velocity_prepare(s->s3f, &s->s3_staged))
            s->s3f.staged_v = &s->s3_staged;
        // fused step (both half-steps in one wavefront launch) on top of the
        // staged stress tiles, on request (SEIDART_S3_WAVE=1)
        if (s->s3f.staged && !s->s3f.staged_v && want_wave && s->s3_velocity_kind == S3K_CELL && s->wave_ctl) {
            s->s3f.wave_ctl = s->wave_ctl;
            s->s3f.wave_n = s->wave_n;
            s->s3f.wave_ctas = seismic3_wave_prepare(s->s3f);
            const char* lg = getenv("SEIDART_S3_WAVE_LAG");
            s->s3f.wave_lag = (lg && *lg >= '0' && *lg <= '9') ? atoi(lg) : 0;
            if (cudaMemsetAsync(s->wave_ctl, 0, sizeof(int) * s->wave_n, s->stream) != cudaSuccess ||
                s->s3f.wave_ctas < 1) {
                cudaGetLastError();
                s->s3f.wave_ctl = nullptr;
                s->s3f.wave_n = 0;
            }
        }
        // the staged stress kernel holds the 36 stress-loop C-PML memories as
        // 21 (SEIDART_S3_MERGE=0 keeps all 36); the fused step keeps 36
        const char* mg = getenv("SEIDART_S3_MERGE");
        s->s3f.mem_merged = (s->s3f.staged && !s->s3f.wave_ctl && !(mg && *mg == '0')) ? 1 : 0;
    }
    trace.mark("kernel set-up", s->stream);
    *out = s;
    return SEIDART_OK;
}

int seidart_solver_set_stream(SeidartSolver* s, void* stream) {
    if (!s) return set_err(SEIDART_ERR_ARG, "NULL solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (s->own_stream) cudaStreamDestroy(s->stream);
    for (int q = 0; q < 2; ++q)
        if (s->graph_exec[q]) { cudaGraphExecDestroy(s->graph_exec[q]); s->graph_exec[q] = nullptr; s->graph_len[q] = 0; }
    if (stream) { s->stream = (cudaStream_t)stream; s->own_stream = false; }
    else { CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)); s->own_stream = true; }
    return SEIDART_OK;
}

int seidart_solver_set_fields(SeidartSolver* s, const double* const* fields) {
    if (!s || !fields) return set_err(SEIDART_ERR_ARG, "NULL argument");
    const size_t n = s->ncell * (s->L.cplx ? 2 : 1);
    for (int q = 0; q < s->L.nfield; ++q) {
        if (!fields[q]) continue;  // NULL keeps the current values
        const int rc = s->precision == SEIDART_FP32 ? upload<float>(*s, s->fields[q], fields[q], n)
                                                    : upload<double>(*s, s->fields[q], fields[q], n);
        if (rc != SEIDART_OK) return rc;
    }
    return SEIDART_OK;
}

static int zero_rings(SeidartSolver* s) {
    // electromag2: the Hy ring is zeroed lazily by the next H update
    if (s->family == SEIDART_ELECTROMAG2) {
        const int per = 2 * s->dom.nx + 2 * s->dom.nz;
        if (s->precision == SEIDART_FP32)
            zero_ring2d<float><<<(per + 255) / 256, 256, 0, s->stream>>>((float*)s->fields[E2_HY], s->dom.nx, s->dom.nz, 1);
        else
            zero_ring2d<double><<<(per + 255) / 256, 256, 0, s->stream>>>((double*)s->fields[E2_HY], s->dom.nx, s->dom.nz, 1);
        CUDA_TRY(cudaGetLastError());
    }
    // electromag3: the six H faces are zeroed lazily by the next H update
    if (s->family == SEIDART_ELECTROMAG3) {
        for (int q = E3_HX; q <= E3_HZ; ++q) {
            if (s->precision == SEIDART_FP32)
                zero_faces3d<float><<<4 * 152, 256, 0, s->stream>>>((float*)s->fields[q], s->dom.nx, s->dom.ny, s->dom.nz);
            else
                zero_faces3d<double><<<4 * 152, 256, 0, s->stream>>>((double*)s->fields[q], s->dom.nx, s->dom.ny, s->dom.nz);
        }
        CUDA_TRY(cudaGetLastError());
    }
    return SEIDART_OK;
}

int seidart_solver_get_fields(SeidartSolver* s, double* const* fields) {
    if (!s || !fields) return set_err(SEIDART_ERR_ARG, "NULL argument");
    int rc = zero_rings(s);
    if (rc != SEIDART_OK) return rc;
    const size_t n = s->ncell * (s->L.cplx ? 2 : 1);
    for (int q = 0; q < s->L.nfield; ++q) {
        if (!fields[q]) continue;
        rc = s->precision == SEIDART_FP32 ? download<float>(*s, fields[q], s->fields[q], n)
                                          : download<double>(*s, fields[q], s->fields[q], n);
        if (rc != SEIDART_OK) return rc;
    }
    return SEIDART_OK;
}

int seidart_solver_get_memory(SeidartSolver* s, double* const* mem) {
    if (!s || !mem) return set_err(SEIDART_ERR_ARG, "NULL argument");
    const size_t n = s->ncell * (s->L.cplx ? 2 : 1);
    float* tmp = nullptr;  // a rebuilt stress-loop memory of the merged layout
    for (int q = 0; q < s->L.nmem; ++q) {
        if (!mem[q]) continue;
        const void* src = s->mem[q];
        if (s->family == SEIDART_SEISMIC3 && s->precision == SEIDART_FP32 && s->s3f.mem_merged && q < 36) {
            if (!tmp && cudaMalloc((void**)&tmp, n * sizeof(float)) != cudaSuccess) {
                cudaGetLastError();
                return set_err(SEIDART_ERR_NOMEM, "no device memory to rebuild the C-PML memories");
            }
            s3_unmerge<<<4 * 152, 256, 0, s->stream>>>(s->s3f, q, tmp);
            src = tmp;
        }
        const int rc = s->precision == SEIDART_FP32 ? download<float>(*s, mem[q], src, n)
                                                    : download<double>(*s, mem[q], src, n);
        if (rc != SEIDART_OK) {
            if (tmp) cudaFree(tmp);
            return rc;
        }
    }
    if (tmp) cudaFree(tmp);
    return SEIDART_OK;
}

int seidart_solver_step(SeidartSolver* s, int nsteps) {
    seidart_trace::Range nvtx("seidart_solver_step");
    if (!s) return set_err(SEIDART_ERR_ARG, "NULL solver");
    if (nsteps < 0 || s->steps_done + nsteps > s->src.time_steps)
        return set_err(SEIDART_ERR_ARG, "stepping %d steps from step %d exceeds time_steps = %d", nsteps,
                       s->steps_done, s->src.time_steps);
    const int chunk = (s->family == SEIDART_SEISMIC3 || s->family == SEIDART_ELECTROMAG3) ? 16 : 64;
    int left = nsteps;
    while (left > 0) {
        const int len = left >= chunk ? chunk : left;
        cudaGraphExec_t ex = nullptr;
        if (s->graphs_ok && graph_for(*s, len, &ex) == SEIDART_OK) {
            CUDA_TRY(cudaGraphLaunch(ex, s->stream));
        } else {
            // streams that cannot be captured (the legacy default stream) launch directly
            cudaGetLastError();
            s->graphs_ok = false;
            for (int t = 0; t < len; ++t) launch_one_step(*s, s->stream);
            CUDA_TRY(cudaGetLastError());
        }
        left -= len;
    }
    s->steps_done += nsteps;
    s->launches = (long long)nsteps * launches_per_step(*s);
    return SEIDART_OK;
}

int seidart_solver_sync(SeidartSolver* s) {
    seidart_trace::Range nvtx("seidart_solver_sync");
    if (!s) return set_err(SEIDART_ERR_ARG, "NULL solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    CUDA_TRY(cudaGetLastError());
    if (s->err_dev) {
        int err = 0;
        CUDA_TRY(cudaMemcpy(&err, s->err_dev, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) {
            // report it once: clear the word so later steps start clean
            CUDA_TRY(cudaMemset(s->err_dev, 0, sizeof(int)));
            return set_err(SEIDART_ERR_TIMEOUT, "a bounded device wait (copy or plane wait) did not complete");
        }
    }
    if (s->steps_done == 0) return SEIDART_OK;
    std::vector<double> nrm(s->steps_done);
    CUDA_TRY(cudaMemcpy(nrm.data(), s->norms, sizeof(double) * s->steps_done, cudaMemcpyDeviceToHost));
    for (int t = 0; t < s->steps_done; ++t)
        if (!(nrm[t] <= 1.0e25))  // > threshold, or NaN
            return set_err(SEIDART_ERR_UNSTABLE, "code became unstable and blew up at step %d (max |v| = %g)", t + 1, nrm[t]);
    return SEIDART_OK;
}

int seidart_solver_traces(SeidartSolver* s, double* traces, double* norms) {
    if (!s) return set_err(SEIDART_ERR_ARG, "NULL solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    const size_t per = (size_t)s->L.ncomp * s->nrec * (s->L.cplx ? 2 : 1);
    if (traces && s->nrec > 0) {
        const int rc = s->precision == SEIDART_FP32 ? download<float>(*s, traces, s->traces, per * s->steps_done)
                                                    : download<double>(*s, traces, s->traces, per * s->steps_done);
        if (rc != SEIDART_OK) return rc;
    }
    if (norms) {
        for (int q = 0; q < s->nnorm; ++q)
            CUDA_TRY(cudaMemcpy(norms + (size_t)q * s->steps_done, s->norms + (size_t)q * s->src.time_steps,
                                sizeof(double) * s->steps_done, cudaMemcpyDeviceToHost));
    }
    return SEIDART_OK;
}

int seidart_solver_profile(SeidartSolver* s, int nsteps, double* total_ms, double* kernel_ms, int* kernel_launches,
                           char* names, int names_len) {
    if (!s || nsteps < 1) return set_err(SEIDART_ERR_ARG, "bad arguments");
    if (s->steps_done + nsteps > s->src.time_steps)
        return set_err(SEIDART_ERR_ARG, "stepping %d steps from step %d exceeds time_steps = %d", nsteps,
                       s->steps_done, s->src.time_steps);
    const int per = 8;
    EventLog L;
    L.st = s->stream;
    L.ev.resize((size_t)nsteps * per + 1);
    L.kid.assign(L.ev.size(), -1);
    for (auto& e : L.ev) CUDA_TRY(cudaEventCreate(&e));
    CUDA_TRY(cudaEventRecord(L.ev[0], s->stream));
    L.next = 1;
    LaunchHook h{&EventLog::on_launch, &L};
    for (int t = 0; t < nsteps; ++t) launch_one_step(*s, s->stream, &h);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    double km[per] = {0}; int kl[per] = {0};
    float tot = 0.f;
    if (e == cudaSuccess && !L.failed) {
        for (size_t q = 1; q < L.next; ++q) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, L.ev[q - 1], L.ev[q]);
            const int k = L.kid[q];
            if (k >= 0 && k < per) { km[k] += ms; kl[k] += 1; }
        }
        cudaEventElapsedTime(&tot, L.ev[0], L.ev[L.next - 1]);
    }
    for (auto& ev : L.ev) cudaEventDestroy(ev);
    if (e != cudaSuccess) return set_err(SEIDART_ERR_CUDA, "profile run failed: %s", cudaGetErrorString(e));
    if (L.failed) return set_err(SEIDART_ERR_CUDA, "profile event recording failed");
    s->steps_done += nsteps;
    s->launches = 0;
    for (int k = 0; k < per; ++k) s->launches += kl[k];
    if (total_ms) *total_ms = tot;
    for (int k = 0; k < per; ++k) {
        if (kernel_ms) kernel_ms[k] = km[k];
        if (kernel_launches) kernel_launches[k] = kl[k];
        if (names && names_len > 0) {
            const std::string nm = k < (int)L.names.size() ? L.names[k] : std::string();
            snprintf(names + (size_t)k * names_len, names_len, "%s", nm.c_str());
        }
    }
    return SEIDART_OK;
}

int seidart_solver_steps_done(const SeidartSolver* s) { return s ? s->steps_done : -1; }

int seidart_solver_material_count(const SeidartSolver* s) { return s ? s->s3_nmat : -1; }

int seidart_solver_cpml_tuples(const SeidartSolver* s) { return s ? s->s3_ncpml : -1; }

int seidart_solver_stress_memory_arrays(const SeidartSolver* s) {
    if (!s) return -1;
    if (s->family != SEIDART_SEISMIC3) return 0;
    return (s->precision == SEIDART_FP32 && s->s3f.mem_merged) ? 21 : 36;
}

int seidart_solver_snapshot_source(SeidartSolver* s, int slot, void** dev, int* is_complex, int* is_fp32,
                                   size_t* ncell, void** stream) {
    if (!s || slot < 0 || slot >= (int)s->fields.size()) return set_err(SEIDART_ERR_ARG, "bad field slot");
    if (dev) *dev = s->fields[slot];
    if (is_complex) *is_complex = s->L.cplx;
    if (is_fp32) *is_fp32 = s->precision == SEIDART_FP32;
    if (ncell) *ncell = s->ncell;
    if (stream) *stream = (void*)s->stream;
    return SEIDART_OK;
}

void* seidart_solver_field_ptr(SeidartSolver* s, int slot) {
    if (!s || slot < 0 || slot >= (int)s->fields.size()) return nullptr;
    return s->fields[slot];
}

long long seidart_solver_launches(const SeidartSolver* s) { return s ? s->launches : -1; }

int seidart_solver_set_wait(SeidartSolver* s, int limit, int probe_bytes) {
    if (!s) return set_err(SEIDART_ERR_ARG, "NULL solver");
    if (limit < 1 || probe_bytes < 0 || probe_bytes % 16 != 0)
        return set_err(SEIDART_ERR_ARG, "wait limit must be >= 1 and probe bytes a non-negative multiple of 16");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->s3f.wait_limit = limit;
    s->s3f.wait_probe = probe_bytes;
    // the launch arguments are baked into the captured step graphs
    for (int q = 0; q < 2; ++q)
        if (s->graph_exec[q]) { cudaGraphExecDestroy(s->graph_exec[q]); s->graph_exec[q] = nullptr; s->graph_len[q] = 0; }
    return SEIDART_OK;
}

int seidart_solver_destroy(SeidartSolver* s) {
    if (!s) return SEIDART_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (int q = 0; q < 2; ++q)
        if (s->graph_exec[q]) cudaGraphExecDestroy(s->graph_exec[q]);
    if (s->arena) cudaFree(s->arena);
    if (s->s3_packed) cudaFree(s->s3_packed);
    if (s->s3_mat_ids) cudaFree(s->s3_mat_ids);
    if (s->s3_mat_tab) cudaFree(s->s3_mat_tab);
    if (s->s3_cpml_ids) cudaFree(s->s3_cpml_ids);
    if (s->s3_cpml_tab) cudaFree(s->s3_cpml_tab);
    if (s->stage) cudaFree(s->stage);
    if (s->pin) cudaFreeHost(s->pin);
    for (int b = 0; b < 2; ++b)
        if (s->pin_ev[b]) cudaEventDestroy(s->pin_ev[b]);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SEIDART_OK;
}

// ---- internal hooks for the batched runtime (batch.cu); not part of the ABI
int seidart_solver_internal_s2f(SeidartSolver* s, S2Args<float>* out, const int** rec) {
    if (!s || s->family != SEIDART_SEISMIC2 || s->precision != SEIDART_FP32) return set_err(SEIDART_ERR_ARG, "not an FP32 seismic2 solver");
    *out = s->s2f;
    if (rec) *rec = s->rec_dev;
    return SEIDART_OK;
}

int seidart_solver_internal_e2f(SeidartSolver* s, E2Args<float>* out, const int** rec) {
    if (!s || s->family != SEIDART_ELECTROMAG2 || s->precision != SEIDART_FP32) return set_err(SEIDART_ERR_ARG, "not an FP32 electromag2 solver");
    *out = s->e2f;
    if (rec) *rec = s->rec_dev;
    return SEIDART_OK;
}

// Point dst's read-only model arrays (coefficients, density, attenuation,
// C-PML profiles) at src's, so solvers of one model (the concurrent shots of
// a misfit gradient) read one copy and keep it in L2 together.  Both must be
// FP32 solvers of the same family, grid and model; dst's cached graphs are
// dropped (they hold the launch arguments by value).  dst's own copy stays
// allocated but unused.
int seidart_solver_internal_share_model(SeidartSolver* dst, const SeidartSolver* src) {
    if (!dst || !src || dst->family != src->family || dst->precision != SEIDART_FP32 ||
        src->precision != SEIDART_FP32 || dst->ncell != src->ncell)
        return set_err(SEIDART_ERR_ARG, "model sharing needs two FP32 solvers of one family and grid");
    if (dst->family == SEIDART_SEISMIC2) {
        for (int q = 0; q < 16; ++q) dst->s2f.m[q] = src->s2f.m[q];
    } else if (dst->family == SEIDART_ELECTROMAG2) {
        for (int q = 0; q < 10; ++q) dst->e2f.c[q] = src->e2f.c[q];
        for (int q = 0; q < 6; ++q) dst->e2f.cpml[q] = src->e2f.cpml[q];
    } else {
        return set_err(SEIDART_ERR_UNSUPPORTED, "model sharing covers seismic2 and electromag2");
    }
    CUDA_TRY(cudaStreamSynchronize(dst->stream));
    for (int q = 0; q < 2; ++q)
        if (dst->graph_exec[q]) {
            cudaGraphExecDestroy(dst->graph_exec[q]);
            dst->graph_exec[q] = nullptr;
            dst->graph_len[q] = 0;
        }
    return SEIDART_OK;
}

// zero fields, memories, traces and norms; back to step 1
int seidart_solver_internal_reset(SeidartSolver* s) {
    if (!s) return set_err(SEIDART_ERR_ARG, "NULL solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    const size_t n = s->ncell * (s->L.cplx ? 2 : 1) * s->esize;
    for (void* f : s->fields) CUDA_TRY(cudaMemsetAsync(f, 0, n, s->stream));
    for (void* m : s->mem) CUDA_TRY(cudaMemsetAsync(m, 0, n, s->stream));
    const size_t tr = (size_t)s->src.time_steps * s->L.ncomp * (s->nrec > 0 ? s->nrec : 1) * (s->L.cplx ? 2 : 1) * s->esize;
    CUDA_TRY(cudaMemsetAsync(s->traces, 0, tr, s->stream));
    CUDA_TRY(cudaMemsetAsync(s->norms, 0, sizeof(double) * s->src.time_steps * s->nnorm, s->stream));
    const int one = 1;
    CUDA_TRY(cudaMemcpyAsync(s->step_dev, &one, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->steps_done = 0;
    return SEIDART_OK;
}

// account for steps advanced by another runtime on this solver's state
int seidart_solver_internal_advance(SeidartSolver* s, int nsteps) {
    if (!s) return set_err(SEIDART_ERR_ARG, "NULL solver");
    s->steps_done += nsteps;
    return SEIDART_OK;
}

// position the step counter (next step to compute = steps_done + 1)
int seidart_solver_internal_set_step(SeidartSolver* s, int steps_done) {
    if (!s || steps_done < 0 || steps_done > s->src.time_steps) return set_err(SEIDART_ERR_ARG, "bad step");
    const int next = steps_done + 1;
    CUDA_TRY(cudaMemcpyAsync(s->step_dev, &next, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->steps_done = steps_done;
    return SEIDART_OK;
}

// move the point source of an FP32 seismic2 solver (0-based cell) and point
// its vertical-force series at device memory; cached graphs are dropped
// because they hold the launch arguments by value
int seidart_solver_set_plane_wave(SeidartSolver* s, const SeidartPlaneWave* in, const double* const* model) {
    if (!s || !in) return set_err(SEIDART_ERR_ARG, "NULL argument");
    PwDev pw{};
    if (in->kind != 0) {
        if (in->kind != SEIDART_PW_S && in->kind != SEIDART_PW_P) return set_err(SEIDART_ERR_ARG, "unknown plane-wave kind %d", in->kind);
        if (!model) return set_err(SEIDART_ERR_ARG, "the plane-wave set-up needs the host model");
        for (int q = 0; q < s->L.nmodel; ++q)
            if (!model[q]) return set_err(SEIDART_ERR_ARG, "model array %d is NULL", q);
        std::string why;
        const int rc = pw_setup(s->family, &s->dom, &s->src, in, model, &pw, why);
        if (rc != SEIDART_OK) return set_err(rc, "%s", why.c_str());
    }
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    // point-source series are not applied while a plane wave is on
    // (electromag25 keeps its point source, cpmlfdtd.f08:3261-3266)
    const bool drop = pw.on != 0;
    auto apply = [&](auto& a, int nsrc) {
        a.pw = pw;
        if (drop)
            for (int q = 0; q < nsrc; ++q) a.src[q] = nullptr;
    };
    switch (s->family) {
    case SEIDART_SEISMIC2: apply(s->s2d, S2_NSRC); apply(s->s2f, S2_NSRC); break;
    case SEIDART_SEISMIC25: apply(s->s25d, 9); apply(s->s25f, 9); break;
    case SEIDART_SEISMIC3: apply(s->s3d, 9); apply(s->s3f, 9); break;
    case SEIDART_ELECTROMAG2: apply(s->e2d, E2_NSRC); apply(s->e2f, E2_NSRC); break;
    case SEIDART_ELECTROMAG3: apply(s->e3d, E3_NSRC); apply(s->e3f, E3_NSRC); break;
    default: break;  // electromag25: set up, never injected
    }
    if (drop && (s->family == SEIDART_SEISMIC2 || s->family == SEIDART_SEISMIC25 || s->family == SEIDART_SEISMIC3)) {
        s->stress_src = 0;
        s->s2d.stress_src = s->s2f.stress_src = 0;
        s->s25d.stress_src = s->s25f.stress_src = 0;
        s->s3d.stress_src = s->s3f.stress_src = 0;
    }
    for (int q = 0; q < 2; ++q)
        if (s->graph_exec[q]) { cudaGraphExecDestroy(s->graph_exec[q]); s->graph_exec[q] = nullptr; s->graph_len[q] = 0; }
    return SEIDART_OK;
}

int seidart_solver_internal_set_source(SeidartSolver* s, int isrc, int jsrc, const double* dev_srcx,
                                       const double* dev_srcz) {
    if (!s || (s->family != SEIDART_SEISMIC2 && s->family != SEIDART_ELECTROMAG2) || s->precision != SEIDART_FP32)
        return set_err(SEIDART_ERR_ARG, "bad solver");
    if (isrc < 0 || isrc + 1 >= s->dom.nx || jsrc < 0 || jsrc + 1 >= s->dom.nz) return set_err(SEIDART_ERR_ARG, "source outside grid");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (s->family == SEIDART_SEISMIC2) {
        s->s2f.isrc = isrc;
        s->s2f.jsrc = jsrc;
        s->s2f.src[S2_SRCX] = dev_srcx;
        s->s2f.src[S2_SRCZ] = dev_srcz;
    } else {
        s->e2f.isrc = isrc;
        s->e2f.jsrc = jsrc;
        s->e2f.src[E2_SRCX] = dev_srcx;
        s->e2f.src[E2_SRCZ] = dev_srcz;
    }
    for (int q = 0; q < 2; ++q)
        if (s->graph_exec[q]) { cudaGraphExecDestroy(s->graph_exec[q]); s->graph_exec[q] = nullptr; s->graph_len[q] = 0; }
    return SEIDART_OK;
}

cudaStream_t seidart_solver_internal_stream(SeidartSolver* s) { return s ? s->stream : nullptr; }
void* seidart_solver_internal_mem(SeidartSolver* s, int slot) {
    return (s && slot >= 0 && slot < (int)s->mem.size()) ? s->mem[slot] : nullptr;
}
const void* seidart_solver_internal_traces(SeidartSolver* s) { return s ? s->traces : nullptr; }
BoxH seidart_solver_internal_box(SeidartSolver* s) { return s ? s->box : BoxH{}; }
// the per-step launch description (device step counter, receivers) for
// callers that launch the family's kernels themselves (FWI recompute graphs)
StepInfo seidart_solver_internal_stepinfo(SeidartSolver* s) {
    return s ? StepInfo{s->step_dev, s->nrec, s->rec_dev} : StepInfo{nullptr, 0, nullptr};
}

int seidart_run(int family, int precision, const SeidartDomain* dom, const SeidartSource* src, int density_code,
                const double* const* model, const double* const* srcfn, double* const* fields, int nrec,
                const int* rec_cells, double* traces, double* norms) {
    SeidartSolver* s = nullptr;
    int rc = seidart_solver_create(&s, family, precision, dom, src, density_code, model, srcfn, nrec, rec_cells);
    if (rc != SEIDART_OK) return rc;
    if (fields) rc = seidart_solver_set_fields(s, fields);
    if (rc == SEIDART_OK) rc = seidart_solver_step(s, src->time_steps);
    int sync_rc = rc == SEIDART_OK ? seidart_solver_sync(s) : rc;
    std::string err = g_err;
    if (rc == SEIDART_OK && fields) rc = seidart_solver_get_fields(s, fields);
    if (rc == SEIDART_OK) rc = seidart_solver_traces(s, traces, norms);
    seidart_solver_destroy(s);
    if (rc != SEIDART_OK) return rc;
    if (sync_rc != SEIDART_OK) { g_err = err; return sync_rc; }
    return SEIDART_OK;
}

}  // extern "C"
