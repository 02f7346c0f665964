// fileio.cu -- the reference's file contract on top of the GPU solvers.
//
// Inputs are read from a working directory exactly as the reference reads
// them (src/fortran/seidartio.f08:161-292): one Fortran sequential-unformatted
// record per file (4-byte length markers around the payload, FP64 grids in
// column-major order, complex128 for 2.5D initial conditions).  Outputs are
// the per-step snapshots of write_image2 / write_image3
// (src/fortran/seidartio.f08:366-426): `Vx.<it:06d>.<xind>.<zind>.dat`
// (3D: `.<xind>.<yind>.<zind>`), one float32 record unless SINGLE_OUTPUT is
// false, plus velocity_norm.dat / stress_norm.dat for 3D (:186-200).
//
// Snapshot pipeline: after every step a conversion kernel copies the output
// fields into a device ring slot (float32 or float64, real part for 2.5D);
// the ring is drained to pinned host memory on a second stream and a writer
// thread writes the files, so disk I/O overlaps the following steps.
//
// The 2.5D solvers write zstd blocks by default (src/fortran/seidartio.f08:
// 462-734, cpmlfdtd.f08:1295-1318, :3313-3336): the real parts of the three
// output components, CPML stripped, float32, laid out (x, 1, z, component,
// step) for up to steps_per_block steps per file
// `S25.<first:06d>-<last:06d>.<xind>.<yind>.<zind>.blk.zst` (EM25. for
// electromag25); FDTD_LEGACY_OUTPUT=TRUE selects the per-step files instead
// and FDTD_STEPS_PER_BLOCK overrides the block length (default: about 2 GiB
// of float32 per block, at most 500 steps).  A device kernel gathers each
// step into a device block buffer; a full block is copied to pinned host
// memory in one transfer and compressed and written by the writer thread
// while the next block fills (two buffers).  Frames are compressed at level
// 3 by the system libzstd when it can be loaded, else written as a valid
// zstd frame of raw (stored) blocks, which every zstd decoder reads.
//
// Entry points: seidart_run_files (directory + Domain/Source, the body of
// the reference's seismic2/25/3 and electromag2/25 subroutines), the legacy
// C names seismic2_ ... electromag25c_ (legacy/cpmlfdtd_wrapper.c:7-16), and
// seidart_cli_main, the `seidartfdtd <input.json> [seismic=..]
// [density_method=..]` driver of src/fortran/main.f08.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/seidart_gpu.h"
#include "trace.h"

// solver internals used here (defined in solver.cu)
extern "C" int seidart_solver_snapshot_source(SeidartSolver* s, int slot, void** dev, int* is_complex,
                                              int* is_fp32, size_t* ncell, void** stream);

extern "C" int seidart_internal_set_error(int code, const char* msg);

namespace {

std::string g_io_err;
int io_err(int code, const std::string& msg) {
    g_io_err = msg;
    fprintf(stderr, "seidart: %s\n", msg.c_str());
    return code;
}

// ------------------------------------------------------------ Fortran records
// gfortran sequential-unformatted: [int32 n][n bytes][int32 n]; payloads over
// 2^31-9 bytes are split into subrecords whose head marker is negative when
// another subrecord follows.
bool read_record(const std::string& path, std::vector<char>& out, std::string& why) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) { why = "cannot open " + path + ": " + strerror(errno); return false; }
    out.clear();
    for (;;) {
        int32_t head = 0, tail = 0;
        if (fread(&head, 4, 1, f) != 1) { fclose(f); why = path + ": truncated record marker"; return false; }
        const size_t n = (size_t)(head < 0 ? -(int64_t)head : head);
        const size_t off = out.size();
        out.resize(off + n);
        if (n && fread(out.data() + off, 1, n, f) != n) { fclose(f); why = path + ": truncated record"; return false; }
        if (fread(&tail, 4, 1, f) != 1) { fclose(f); why = path + ": missing trailing marker"; return false; }
        if (head >= 0) break;
    }
    fclose(f);
    return true;
}

bool write_record(const std::string& path, const void* data, size_t bytes, std::string& why) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { why = "cannot create " + path + ": " + strerror(errno); return false; }
    const size_t kMax = 2147483639u;
    const char* p = (const char*)data;
    size_t left = bytes;
    bool first = true;
    bool ok = true;
    do {
        const size_t n = left > kMax ? kMax : left;
        const bool more = left > n;
        const int32_t head = more ? -(int32_t)n : (int32_t)n;
        const int32_t tail = first ? (int32_t)n : -(int32_t)n;
        ok = ok && fwrite(&head, 4, 1, f) == 1 && (n == 0 || fwrite(p, 1, n, f) == n) && fwrite(&tail, 4, 1, f) == 1;
        p += n; left -= n; first = false;
    } while (left > 0 && ok);
    if (fclose(f) != 0) ok = false;
    if (!ok) why = "write failed: " + path;
    return ok;
}

// ------------------------------------------------------------------ JSON
// Minimal reader for the reference's input.json (objects, arrays, strings,
// numbers, true/false/null); values are addressed by dotted paths.
struct JsonReader {
    const char* p;
    std::map<std::string, std::string> vals;
    bool ok = true;
    void ws() { while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p; }
    std::string str() {
        std::string s;
        ++p;  // opening quote
        while (*p && *p != '"') {
            if (*p == '\\' && p[1]) { ++p; s += (*p == 'n') ? '\n' : (*p == 't') ? '\t' : *p; ++p; }
            else s += *p++;
        }
        if (*p == '"') ++p; else ok = false;
        return s;
    }
    void value(const std::string& path) {
        ws();
        if (*p == '{') {
            ++p; ws();
            if (*p == '}') { ++p; return; }
            for (;;) {
                ws();
                if (*p != '"') { ok = false; return; }
                const std::string k = str();
                ws();
                if (*p != ':') { ok = false; return; }
                ++p;
                value(path.empty() ? k : path + "." + k);
                if (!ok) return;
                ws();
                if (*p == ',') { ++p; continue; }
                if (*p == '}') { ++p; return; }
                ok = false; return;
            }
        } else if (*p == '[') {
            ++p; ws();
            int idx = 0;
            if (*p == ']') { ++p; return; }
            for (;;) {
                value(path + "[" + std::to_string(idx++) + "]");
                if (!ok) return;
                ws();
                if (*p == ',') { ++p; continue; }
                if (*p == ']') { ++p; return; }
                ok = false; return;
            }
        } else if (*p == '"') {
            vals[path] = str();
        } else {
            const char* b = p;
            while (*p && *p != ',' && *p != '}' && *p != ']' && *p != ' ' && *p != '\n' && *p != '\r' && *p != '\t') ++p;
            if (p == b) { ok = false; return; }
            vals[path] = std::string(b, p);
        }
    }
    bool num(const std::string& k, double& v) const {
        auto it = vals.find(k);
        if (it == vals.end()) return false;
        char* e = nullptr;
        v = strtod(it->second.c_str(), &e);
        return e && *e == 0;
    }
    std::string text(const std::string& k) const {
        auto it = vals.find(k);
        return it == vals.end() ? std::string() : it->second;
    }
};

std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// ------------------------------------------------------------ zstd frames
// libzstd's one-shot API, loaded at run time when present
struct ZstdLib {
    bool tried = false;
    void* h = nullptr;
    size_t (*bound)(size_t) = nullptr;
    size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
    unsigned (*is_error)(size_t) = nullptr;
    bool load() {
        if (tried) return h != nullptr;
        tried = true;
        const char* raw = getenv("SEIDART_ZSTD_RAW");
        if (raw && *raw == '1') return false;
        for (const char* nm : {"libzstd.so.1", "libzstd.so"}) {
            h = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
            if (h) break;
        }
        if (!h) return false;
        bound = (size_t(*)(size_t))dlsym(h, "ZSTD_compressBound");
        compress = (size_t(*)(void*, size_t, const void*, size_t, int))dlsym(h, "ZSTD_compress");
        is_error = (unsigned (*)(size_t))dlsym(h, "ZSTD_isError");
        if (!bound || !compress || !is_error) {
            dlclose(h);
            h = nullptr;
        }
        return h != nullptr;
    }
};
ZstdLib g_zstd;
std::mutex g_zstd_mu;

// One zstd frame (RFC 8878) holding `bytes` of data in raw blocks: magic,
// frame header (8-byte content size, 128 KiB window), then blocks of at most
// 128 KiB, each with a 3-byte header (last-block bit, type 0 = raw, size).
void raw_zstd_frame(const char* data, size_t bytes, std::vector<char>& out) {
    const size_t B = 128 * 1024;
    out.clear();
    out.reserve(bytes + 14 + 3 * (bytes / B + 1));
    const uint8_t head[6] = {0x28, 0xB5, 0x2F, 0xFD, 0xC0, 0x38};  // magic; FCS 8 bytes; window 2^17
    out.insert(out.end(), head, head + 6);
    for (int b = 0; b < 8; ++b) out.push_back((char)((uint64_t)bytes >> (8 * b) & 0xFF));
    size_t off = 0;
    do {
        const size_t n = bytes - off < B ? bytes - off : B;
        const uint32_t last = off + n == bytes ? 1u : 0u;
        const uint32_t hdr = last | (0u << 1) | ((uint32_t)n << 3);
        out.push_back((char)(hdr & 0xFF));
        out.push_back((char)(hdr >> 8 & 0xFF));
        out.push_back((char)(hdr >> 16 & 0xFF));
        out.insert(out.end(), data + off, data + off + n);
        off += n;
    } while (off < bytes);
}

bool write_zst(const std::string& path, const void* data, size_t bytes, std::string& why) {
    std::vector<char> buf;
    bool lib;
    {
        std::lock_guard<std::mutex> lk(g_zstd_mu);
        lib = g_zstd.load();
    }
    if (lib) {
        buf.resize(g_zstd.bound(bytes));
        const size_t n = g_zstd.compress(buf.data(), buf.size(), data, bytes, 3);
        if (g_zstd.is_error(n)) { why = path + ": zstd compression failed"; return false; }
        buf.resize(n);
    } else {
        raw_zstd_frame((const char*)data, bytes, buf);
    }
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { why = "cannot open " + path + ": " + strerror(errno); return false; }
    const bool ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    if (fclose(f) != 0 || !ok) { why = "write failed: " + path; return false; }
    return true;
}

// -------------------------------------------------------------- snapshots
template <typename TI, typename TO>
__global__ void snap_copy(const TI* __restrict__ in, TO* __restrict__ out, size_t n, int stride) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = (TO)in[q * stride];  // stride 2 takes the real part of complex fields
}

struct WriterThread {
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::function<bool()>> q;
    bool stop = false, failed = false;
    std::thread th;
    WriterThread() {
        th = std::thread([this] {
            for (;;) {
                std::function<bool()> job;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [this] { return stop || !q.empty(); });
                    if (q.empty()) return;
                    job = std::move(q.front());
                    q.pop_front();
                }
                const bool ok = job();
                std::lock_guard<std::mutex> lk(mu);
                if (!ok) failed = true;
                cv.notify_all();
            }
        });
    }
    void push(std::function<bool()> f) {
        std::lock_guard<std::mutex> lk(mu);
        q.push_back(std::move(f));
        cv.notify_all();
    }
    void drain() {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [this] { return q.empty(); });
    }
    ~WriterThread() {
        { std::lock_guard<std::mutex> lk(mu); stop = true; cv.notify_all(); }
        th.join();
    }
};

// Output pipeline for `nchan` fields: ring of R device slots -> pinned host.
struct SnapshotPipe {
    SeidartSolver* s = nullptr;
    std::vector<int> slots;
    std::vector<std::string> chans;
    bool single = true;
    size_t ncell = 0, esz = 4;
    int R = 4;
    cudaStream_t comp = nullptr, copy = nullptr;
    std::vector<void*> dring;   // R device slots, each nchan * ncell * esz
    std::vector<void*> hring;   // R pinned host slots
    std::vector<cudaEvent_t> ready, copied;
    std::vector<int> pending_step;
    WriterThread writer;
    std::string name_suffix;
    bool failed = false;
    std::string why;

    int init(SeidartSolver* solver, const std::vector<int>& sl, const std::vector<std::string>& ch, bool sgl,
             const std::string& suffix) {
        s = solver; slots = sl; chans = ch; single = sgl; name_suffix = suffix;
        void* dev; int cplx, f32; void* st;
        if (seidart_solver_snapshot_source(s, slots[0], &dev, &cplx, &f32, &ncell, &st) != SEIDART_OK)
            return io_err(SEIDART_ERR_ARG, "snapshot set-up failed");
        comp = (cudaStream_t)st;
        esz = single ? 4 : 8;
        const size_t bytes = slots.size() * ncell * esz;
        // keep the ring within ~4 GiB of device memory
        R = (int)std::max<size_t>(2, std::min<size_t>(8, (4ull << 30) / std::max<size_t>(bytes, 1)));
        if (cudaStreamCreateWithFlags(&copy, cudaStreamNonBlocking) != cudaSuccess) return io_err(SEIDART_ERR_CUDA, "stream");
        dring.assign(R, nullptr); hring.assign(R, nullptr);
        ready.assign(R, nullptr); copied.assign(R, nullptr); pending_step.assign(R, 0);
        for (int r = 0; r < R; ++r) {
            if (cudaMalloc(&dring[r], bytes) != cudaSuccess || cudaMallocHost(&hring[r], bytes) != cudaSuccess ||
                cudaEventCreateWithFlags(&ready[r], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&copied[r], cudaEventDisableTiming) != cudaSuccess)
                return io_err(SEIDART_ERR_NOMEM, "snapshot ring allocation failed");
        }
        return SEIDART_OK;
    }
    // capture the current fields of step `it` (call right after the step)
    int capture(int it) {
        const int r = (it - 1) % R;
        if (pending_step[r]) {  // slot still in flight: wait for its copy and file writes
            cudaEventSynchronize(copied[r]);
            writer.drain();
            pending_step[r] = 0;
        }
        const size_t bytes1 = ncell * esz;
        for (size_t c = 0; c < slots.size(); ++c) {
            void* dev; int cplx, f32; void* st; size_t n;
            seidart_solver_snapshot_source(s, slots[c], &dev, &cplx, &f32, &n, &st);
            char* dst = (char*)dring[r] + c * bytes1;
            const int stride = cplx ? 2 : 1;
            const int blocks = 4 * 152;
            if (f32 && single) snap_copy<float, float><<<blocks, 256, 0, comp>>>((const float*)dev, (float*)dst, n, stride);
            else if (f32) snap_copy<float, double><<<blocks, 256, 0, comp>>>((const float*)dev, (double*)dst, n, stride);
            else if (single) snap_copy<double, float><<<blocks, 256, 0, comp>>>((const double*)dev, (float*)dst, n, stride);
            else snap_copy<double, double><<<blocks, 256, 0, comp>>>((const double*)dev, (double*)dst, n, stride);
        }
        if (cudaGetLastError() != cudaSuccess) return io_err(SEIDART_ERR_CUDA, "snapshot kernel launch failed");
        if (cudaEventRecord(ready[r], comp) != cudaSuccess || cudaStreamWaitEvent(copy, ready[r], 0) != cudaSuccess ||
            cudaMemcpyAsync(hring[r], dring[r], slots.size() * bytes1, cudaMemcpyDeviceToHost, copy) != cudaSuccess ||
            cudaEventRecord(copied[r], copy) != cudaSuccess)
            return io_err(SEIDART_ERR_CUDA, std::string("snapshot copy could not be issued: ") +
                                                cudaGetErrorString(cudaGetLastError()));
        pending_step[r] = it;
        // writer: wait for this slot's copy, then write one file per channel
        cudaEvent_t ev = copied[r];
        char* host = (char*)hring[r];
        for (size_t c = 0; c < slots.size(); ++c) {
            char name[256];
            snprintf(name, sizeof name, "%s.%06d%s", chans[c].c_str(), it, name_suffix.c_str());
            std::string path = name;
            const char* data = host + c * bytes1;
            writer.push([ev, path, data, bytes1, this]() {
                if (cudaEventSynchronize(ev) != cudaSuccess) return false;
                std::string w;
                if (!write_record(path, data, bytes1, w)) { why = w; return false; }
                return true;
            });
        }
        return SEIDART_OK;
    }
    int finish() {
        cudaStreamSynchronize(copy);
        writer.drain();
        if (writer.failed) return io_err(SEIDART_ERR_IO, why.empty() ? "snapshot write failed" : why);
        return SEIDART_OK;
    }
    ~SnapshotPipe() {
        if (copy) cudaStreamSynchronize(copy);
        writer.drain();
        for (int r = 0; r < (int)dring.size(); ++r) {
            if (dring[r]) cudaFree(dring[r]);
            if (hring[r]) cudaFreeHost(hring[r]);
            if (ready[r]) cudaEventDestroy(ready[r]);
            if (copied[r]) cudaEventDestroy(copied[r]);
        }
        if (copy) cudaStreamDestroy(copy);
    }
};

// Real parts of three 2D fields, CPML stripped, as float32 slabs
// out[c][z][x] (one step of the (x, 1, z, component, step) block).
template <typename T>
__global__ void block_gather(const T* __restrict__ f0, const T* __restrict__ f1, const T* __restrict__ f2,
                             float* __restrict__ out, int nx, int cpml, int onx, int onz, int stride) {
    const size_t slab = (size_t)onx * onz;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < 3 * slab; q += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(q / slab);
        const size_t r = q - (size_t)c * slab;
        const int x = (int)(r % onx), z = (int)(r / onx);
        const size_t src = ((size_t)(x + cpml) + (size_t)nx * (z + cpml)) * stride;
        const T* f = c == 0 ? f0 : (c == 1 ? f1 : f2);
        out[q] = (float)f[src];
    }
}

// zstd block output of the 2.5D solvers (see the file comment)
struct BlockPipe {
    SeidartSolver* s = nullptr;
    std::vector<int> slots;
    std::string prefix;            // "S25." or "EM25." (with the directory)
    int nx = 0, nz = 0, cpml = 0, onx = 0, onz = 0, spb = 1, nt = 0;
    int xind = 0, yind = 0, zind = 0;
    size_t slab = 0;               // onx * onz
    cudaStream_t comp = nullptr, copy = nullptr;
    float* dblk[2] = {nullptr, nullptr};
    float* hblk[2] = {nullptr, nullptr};
    cudaEvent_t full[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    bool busy[2] = {false, false};
    int cur = 0, in_block = 0, block_count = 0;
    WriterThread writer;
    std::string why;

    static int steps_per_block(int onx, int onz) {
        const char* e = getenv("FDTD_STEPS_PER_BLOCK");
        if (e && *e) return std::max(1, atoi(e));
        const double per = (double)onx * onz * 3 * 4;
        int n = std::max(1, (int)(2147483648.0 / per));
        return n > 500 ? 500 : n;
    }
    int init(SeidartSolver* solver, const std::vector<int>& sl, const std::string& pfx, const SeidartDomain* dom,
             const SeidartSource* src) {
        s = solver; slots = sl; prefix = pfx;
        nx = dom->nx; nz = dom->nz; cpml = dom->cpml; nt = src->time_steps;
        xind = src->xind; yind = src->yind; zind = src->zind;
        onx = nx - 2 * cpml; onz = nz - 2 * cpml;
        if (cpml < 0 || onx < 1 || onz < 1) return io_err(SEIDART_ERR_ARG, "cpml removes the entire zstd block output domain");
        slab = (size_t)onx * onz;
        spb = std::min(steps_per_block(onx, onz), std::max(nt, 1));
        void* dev; int cplx, f32; void* st; size_t n;
        if (seidart_solver_snapshot_source(s, slots[0], &dev, &cplx, &f32, &n, &st) != SEIDART_OK)
            return io_err(SEIDART_ERR_ARG, "block output set-up failed");
        comp = (cudaStream_t)st;
        if (cudaStreamCreateWithFlags(&copy, cudaStreamNonBlocking) != cudaSuccess) return io_err(SEIDART_ERR_CUDA, "stream");
        const size_t bytes = 3 * slab * spb * sizeof(float);
        for (int b = 0; b < 2; ++b)
            if (cudaMalloc((void**)&dblk[b], bytes) != cudaSuccess || cudaMallocHost((void**)&hblk[b], bytes) != cudaSuccess ||
                cudaEventCreateWithFlags(&full[b], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming) != cudaSuccess)
                return io_err(SEIDART_ERR_NOMEM, "zstd block buffer allocation failed");
        return SEIDART_OK;
    }
    std::string block_name() const {
        const int ii = (block_count - 1) * spb + 1, jj = std::min(block_count * spb, nt);
        char name[160];
        snprintf(name, sizeof name, "%06d-%06d.%d.%d.%d.blk.zst", ii, jj, xind, yind, zind);
        return prefix + name;
    }
    // hand the current block to the copy stream and the writer; false (and
    // the reason in err) when the copy could not be issued
    bool flush(std::string& err) {
        if (in_block == 0) return true;
        const int b = cur;
        const size_t bytes = 3 * slab * (size_t)in_block * sizeof(float);
        if (cudaEventRecord(full[b], comp) != cudaSuccess || cudaStreamWaitEvent(copy, full[b], 0) != cudaSuccess ||
            cudaMemcpyAsync(hblk[b], dblk[b], bytes, cudaMemcpyDeviceToHost, copy) != cudaSuccess ||
            cudaEventRecord(copied[b], copy) != cudaSuccess) {
            err = std::string("block copy could not be issued: ") + cudaGetErrorString(cudaGetLastError());
            return false;
        }
        busy[b] = true;
        const std::string path = block_name();
        cudaEvent_t ev = copied[b];
        const char* host = (const char*)hblk[b];
        writer.push([this, ev, path, host, bytes]() {
            if (cudaEventSynchronize(ev) != cudaSuccess) { why = "block copy failed"; return false; }
            std::string w;
            if (!write_zst(path, host, bytes, w)) { why = w; return false; }
            return true;
        });
        cur ^= 1;
        in_block = 0;
        return true;
    }
    int capture(int it) {
        (void)it;
        if (in_block == 0) {
            ++block_count;
            if (busy[cur]) {  // the buffer's previous block must be written out first
                writer.drain();
                busy[cur] = false;
            }
        }
        void* dev[3]; int cplx = 0, f32 = 0; void* st; size_t n;
        for (int c = 0; c < 3; ++c) seidart_solver_snapshot_source(s, slots[c], &dev[c], &cplx, &f32, &n, &st);
        float* out = dblk[cur] + 3 * slab * (size_t)in_block;
        const int stride = cplx ? 2 : 1;
        if (f32) block_gather<float><<<4 * 152, 256, 0, comp>>>((const float*)dev[0], (const float*)dev[1], (const float*)dev[2], out, nx, cpml, onx, onz, stride);
        else block_gather<double><<<4 * 152, 256, 0, comp>>>((const double*)dev[0], (const double*)dev[1], (const double*)dev[2], out, nx, cpml, onx, onz, stride);
        if (cudaGetLastError() != cudaSuccess) return io_err(SEIDART_ERR_CUDA, "block gather launch failed");
        std::string err;
        if (++in_block == spb && !flush(err)) return io_err(SEIDART_ERR_CUDA, err);
        return SEIDART_OK;
    }
    int finish() {
        std::string err;
        if (!flush(err)) return io_err(SEIDART_ERR_CUDA, err);
        if (copy) cudaStreamSynchronize(copy);
        writer.drain();
        if (writer.failed) return io_err(SEIDART_ERR_IO, why.empty() ? "zstd block write failed" : why);
        return SEIDART_OK;
    }
    ~BlockPipe() {
        if (copy) cudaStreamSynchronize(copy);
        writer.drain();
        for (int b = 0; b < 2; ++b) {
            if (dblk[b]) cudaFree(dblk[b]);
            if (hblk[b]) cudaFreeHost(hblk[b]);
            if (full[b]) cudaEventDestroy(full[b]);
            if (copied[b]) cudaEventDestroy(copied[b]);
        }
        if (copy) cudaStreamDestroy(copy);
    }
};

// ------------------------------------------------------------ input files
struct Inputs {
    std::vector<std::vector<double>> model, src, fields;
    std::string why;
};

bool load_grid(const std::string& dir, const std::string& name, size_t n, std::vector<double>& out, std::string& why,
               bool optional = false, double fill = 0.0) {
    std::vector<char> rec;
    const std::string path = dir + "/" + name;
    if (!read_record(path, rec, why)) {
        if (optional) { out.assign(n, fill); why.clear(); return true; }
        return false;
    }
    if (rec.size() != n * sizeof(double)) {
        why = path + ": record holds " + std::to_string(rec.size()) + " bytes, expected " +
              std::to_string(n * sizeof(double));
        return false;
    }
    out.resize(n);
    memcpy(out.data(), rec.data(), rec.size());
    return true;
}

}  // namespace

extern "C" {

const char* seidart_io_last_error(void) { return g_io_err.c_str(); }

// one zstd frame of `bytes` (libzstd level 3 when it loads, else raw blocks)
int seidart_zstd_write(const char* path, const void* data, size_t bytes) {
    if (!path || (!data && bytes)) return io_err(SEIDART_ERR_ARG, "NULL argument");
    std::string why;
    if (!write_zst(path, data, bytes, why)) return io_err(SEIDART_ERR_IO, why);
    return SEIDART_OK;
}

// one Fortran record (used by the material pre-pass writers); not part of the ABI
int seidart_internal_write_record(const char* path, const void* data, size_t bytes) {
    std::string why;
    if (!write_record(path, data, bytes, why)) {
        seidart_internal_set_error(SEIDART_ERR_IO, why.c_str());
        return io_err(SEIDART_ERR_IO, why);
    }
    return SEIDART_OK;
}

int seidart_run_files(const char* dir_c, int family, int precision, const SeidartDomain* dom,
                      const SeidartSource* src, int density_code, const char* source_type, int single_output,
                      int write_snapshots) {
    return seidart_run_files_pw(dir_c, family, precision, dom, src, density_code, source_type, single_output,
                                write_snapshots, nullptr);
}

int seidart_run_files_pw(const char* dir_c, int family, int precision, const SeidartDomain* dom,
                         const SeidartSource* src, int density_code, const char* source_type, int single_output,
                         int write_snapshots, const SeidartPlaneWave* pw_in) {
    seidart_trace::Range nvtx("seidart_run_files");
    if (!dom || !src) return io_err(SEIDART_ERR_ARG, "NULL domain/source");
    const std::string dir = dir_c && *dir_c ? dir_c : ".";
    const std::string stype = source_type ? trim(source_type) : std::string("ac");
    // is_plane_wave_source / is_p_wave_source (plane_wave_source.f08:20-36)
    // for the elastic solvers; the EM solvers test source_type == 'pw'
    const bool seis_family = family == SEIDART_SEISMIC2 || family == SEIDART_SEISMIC25 || family == SEIDART_SEISMIC3;
    const bool p_wave = seis_family && (stype == "pwp" || stype == "pw_p" || stype == "pw-p");
    const bool plane = stype == "pw" || (seis_family && (p_wave || stype == "pws" || stype == "pw_s" || stype == "pw-s"));
    if (plane && !pw_in)
        return io_err(SEIDART_ERR_ARG, "source_type \"" + stype + "\" needs the plane-wave parameters");
    int nmodel, nsrc, nfield, nmem, cplx, ncomp;
    if (seidart_layout(family, &nmodel, &nsrc, &nfield, &nmem, &cplx, &ncomp) != SEIDART_OK)
        return io_err(SEIDART_ERR_ARG, "unknown family");
    const bool is3 = family == SEIDART_SEISMIC3 || family == SEIDART_ELECTROMAG3;
    const size_t N = (size_t)dom->nx * (is3 ? dom->ny : 1) * dom->nz;
    const int nt = src->time_steps;
    std::string why;
    std::vector<std::vector<double>> model(nmodel), srcs(nsrc), fields(nfield);
    const char* cpml_files[6] = {"kappa_cpml.dat", "kappa_half_cpml.dat", "acoef_cpml.dat",
                                 "acoef_half_cpml.dat", "bcoef_cpml.dat", "bcoef_half_cpml.dat"};
    std::vector<std::string> mfiles;
    std::vector<std::string> sfiles;
    std::vector<std::string> ffiles;       // initial-condition files per field slot ("" = zero)
    std::vector<int> out_slots;
    std::vector<std::string> out_chans;
    const bool seis = family == SEIDART_SEISMIC2 || family == SEIDART_SEISMIC25 || family == SEIDART_SEISMIC3;
    const bool force = stype == "ac";
    switch (family) {
    case SEIDART_SEISMIC2:
        mfiles = {"c11.dat", "c13.dat", "c15.dat", "c33.dat", "c35.dat", "c55.dat", "rho.dat",
                  "gamma_x.dat", "gamma_z.dat", "gamma_xz.dat"};
        sfiles = {"seismicsourcex.dat", "seismicsourcez.dat", "seismicsourcexx.dat", "seismicsourcexz.dat", "seismicsourcezz.dat"};
        ffiles = {"initialconditionVx.dat", "initialconditionVz.dat", "", "", ""};
        out_slots = {S2_VX, S2_VZ}; out_chans = {"Vx", "Vz"};
        break;
    case SEIDART_SEISMIC25:
    case SEIDART_SEISMIC3: {
        const char* cc[21] = {"c11", "c12", "c13", "c14", "c15", "c16", "c22", "c23", "c24", "c25", "c26",
                              "c33", "c34", "c35", "c36", "c44", "c45", "c46", "c55", "c56", "c66"};
        for (int q = 0; q < 21; ++q) mfiles.push_back(std::string(cc[q]) + ".dat");
        mfiles.push_back("rho.dat");
        for (const char* g : {"gamma_x", "gamma_y", "gamma_z", "gamma_xy", "gamma_yz", "gamma_xz"}) mfiles.push_back(std::string(g) + ".dat");
        sfiles = {"seismicsourcex.dat", "seismicsourcey.dat", "seismicsourcez.dat", "seismicsourcexx.dat",
                  "seismicsourcexy.dat", "seismicsourcexz.dat", "seismicsourceyy.dat", "seismicsourceyz.dat",
                  "seismicsourcezz.dat"};
        ffiles = {"initialconditionVx.dat", "initialconditionVy.dat", "initialconditionVz.dat", "", "", "", "", "", ""};
        out_slots = {S3_VX, S3_VY, S3_VZ}; out_chans = {"Vx", "Vy", "Vz"};
        break;
    }
    case SEIDART_ELECTROMAG2:
        mfiles = {"e11.dat", "e13.dat", "e33.dat", "s11.dat", "s13.dat", "s33.dat"};
        sfiles = {"electromagneticsourcex.dat", "electromagneticsourcez.dat"};
        ffiles = {"initialconditionEx.dat", "initialconditionEz.dat", ""};
        out_slots = {E2_EX, E2_EZ}; out_chans = {"Ex", "Ez"};
        break;
    case SEIDART_ELECTROMAG25:
    case SEIDART_ELECTROMAG3:  // electromag3 reads the same files (cpmlfdtd.f08:3468-3480, :3608-3615)
        mfiles = {"e11.dat", "e12.dat", "e13.dat", "e22.dat", "e23.dat", "e33.dat",
                  "s11.dat", "s12.dat", "s13.dat", "s22.dat", "s23.dat", "s33.dat"};
        sfiles = {"electromagneticsourcex.dat", "electromagneticsourcey.dat", "electromagneticsourcez.dat"};
        ffiles = {"initialconditionEx.dat", "initialconditionEy.dat", "initialconditionEz.dat", "", "", ""};
        out_slots = {E25_EX, E25_EY, E25_EZ}; out_chans = {"Ex", "Ey", "Ez"};
        break;
    }
    for (int q = 0; q < 6; ++q) mfiles.push_back(cpml_files[q]);
    for (int q = 0; q < nmodel; ++q)
        if (!load_grid(dir, mfiles[q], N, model[q], why)) return io_err(SEIDART_ERR_IO, why);
    // sources: 'ac' loads the force components, any other type the stress
    // components (cpmlfdtd.f08:230-237); EM loads the point-source components
    std::vector<const double*> srcp(nsrc, nullptr);
    for (int q = 0; q < nsrc && !plane; ++q) {  // a plane wave loads no source series
        const bool is_force = !seis || q < (family == SEIDART_SEISMIC2 ? 2 : 3);
        if (seis && is_force != force) continue;
        std::vector<char> rec;
        if (!read_record(dir + "/" + sfiles[q], rec, why)) {
            // the reference's 2D solvers do not read a y component
            if (family == SEIDART_SEISMIC2) return io_err(SEIDART_ERR_IO, why);
            return io_err(SEIDART_ERR_IO, why);
        }
        if (rec.size() < (size_t)nt * sizeof(double))
            return io_err(SEIDART_ERR_IO, sfiles[q] + ": fewer than time_steps samples");
        srcs[q].resize(nt);
        memcpy(srcs[q].data(), rec.data(), (size_t)nt * sizeof(double));
        srcp[q] = srcs[q].data();
    }
    std::vector<const double*> mp(nmodel);
    for (int q = 0; q < nmodel; ++q) mp[q] = model[q].data();
    const size_t fn = N * (cplx ? 2 : 1);
    std::vector<const double*> fp(nfield, nullptr);
    for (int q = 0; q < nfield; ++q) {
        if (ffiles[q].empty()) continue;
        if (!load_grid(dir, ffiles[q], fn, fields[q], why)) return io_err(SEIDART_ERR_IO, why);
        fp[q] = fields[q].data();
    }
    SeidartSolver* s = nullptr;
    int rc = seidart_solver_create(&s, family, precision, dom, src, density_code, mp.data(), srcp.data(), 0, nullptr);
    if (rc != SEIDART_OK) return io_err(rc, seidart_last_error());
    rc = seidart_solver_set_fields(s, fp.data());
    if (rc == SEIDART_OK && plane) {
        SeidartPlaneWave pwp = *pw_in;
        pwp.kind = p_wave ? SEIDART_PW_P : SEIDART_PW_S;
        rc = seidart_solver_set_plane_wave(s, &pwp, mp.data());
    }
    if (rc != SEIDART_OK) { seidart_solver_destroy(s); return io_err(rc, seidart_last_error()); }
    char suffix[96];
    if (is3) snprintf(suffix, sizeof suffix, ".%d.%d.%d.dat", src->xind, src->yind, src->zind);
    else snprintf(suffix, sizeof suffix, ".%d.%d.dat", src->xind, src->zind);
    {
        // 2.5D: zstd blocks unless FDTD_LEGACY_OUTPUT=TRUE (seidartio.f08:685-735)
        const char* legacy_env = getenv("FDTD_LEGACY_OUTPUT");
        const bool blocks = write_snapshots && (family == SEIDART_SEISMIC25 || family == SEIDART_ELECTROMAG25) &&
                            !(legacy_env && strcmp(legacy_env, "TRUE") == 0);
        const bool per_step = write_snapshots && !blocks;
        const std::string dirpfx = dir == "." ? std::string() : dir + "/";
        SnapshotPipe pipe;
        BlockPipe bpipe;
        if (per_step) {
            // output paths are relative to the working directory like the reference
            std::string sfx = suffix;
            for (auto& c : out_chans) c = dirpfx + c;
            rc = pipe.init(s, out_slots, out_chans, single_output != 0, sfx);
            if (rc != SEIDART_OK) { seidart_solver_destroy(s); return rc; }
        }
        if (blocks) {
            rc = bpipe.init(s, out_slots, dirpfx + (family == SEIDART_SEISMIC25 ? "S25." : "EM25."), dom, src);
            if (rc != SEIDART_OK) { seidart_solver_destroy(s); return rc; }
        }
        for (int it = 1; it <= nt && rc == SEIDART_OK; ++it) {
            rc = seidart_solver_step(s, 1);
            if (rc == SEIDART_OK && per_step) rc = pipe.capture(it);
            if (rc == SEIDART_OK && blocks) rc = bpipe.capture(it);
            // check the blow-up norm every 64 steps (the reference checks every step and stops)
            if (rc == SEIDART_OK && (it % 64 == 0 || it == nt)) rc = seidart_solver_sync(s);
        }
        int frc = per_step ? pipe.finish() : SEIDART_OK;
        if (blocks && frc == SEIDART_OK) frc = bpipe.finish();
        if (rc == SEIDART_OK) rc = frc;
    }
    if (rc == SEIDART_OK && family == SEIDART_SEISMIC3) {
        // velocity_norm.dat and stress_norm.dat (cpmlfdtd.f08:2282-2283)
        std::vector<double> nrm(2 * (size_t)nt);
        rc = seidart_solver_traces(s, nullptr, nrm.data());
        std::string w;
        if (rc == SEIDART_OK && (!write_record(dir + "/velocity_norm.dat", nrm.data(), nt * sizeof(double), w) ||
                                 !write_record(dir + "/stress_norm.dat", nrm.data() + nt, nt * sizeof(double), w)))
            rc = io_err(SEIDART_ERR_IO, w);
    }
    std::string err = rc == SEIDART_OK ? std::string() : std::string(seidart_last_error());
    seidart_solver_destroy(s);
    if (rc != SEIDART_OK && g_io_err.empty()) g_io_err = err;
    return rc;
}

// ------------------------------------------------- legacy C entry points
// Argument layout of legacy/cpmlfdtd_wrapper.c:7-16: padded nx, nz (ny),
// spacings, PML thickness, src = interior source indices (x, z) or (x, y, z),
// number of steps, single-precision output flag.  Inputs come from the
// working directory.  The legacy layout has no time step: it is derived from
// the model with the legacy rules, dt = min(h)/sqrt(3 max(c11/rho, c33/rho))
// for the 2D elastic solver (legacy/cpmlfdtd_cbindings.f95:867-868),
// 0.7 min(h)/sqrt(3 max(c11/rho, c22/rho, c33/rho)) for the 3D one (:1227-1228)
// and dt = min(h)/(2 c/sqrt(min eps)) for the EM solvers (:2302).
static int legacy_dt(const std::string& dir, int family, size_t N, double hmin, double* dt) {
    std::string why;
    std::vector<double> a, b, r;
    if (family == SEIDART_SEISMIC2 || family == SEIDART_SEISMIC25) {
        if (!load_grid(dir, "c11.dat", N, a, why) || !load_grid(dir, "c33.dat", N, b, why) ||
            !load_grid(dir, "rho.dat", N, r, why))
            return io_err(SEIDART_ERR_IO, why);
        double m = 0.0;
        for (size_t q = 0; q < N; ++q) m = fmax(m, fmax(a[q] / r[q], b[q] / r[q]));
        *dt = hmin / sqrt(3.0 * m);
    } else if (family == SEIDART_SEISMIC3) {
        std::vector<double> c22;
        if (!load_grid(dir, "c11.dat", N, a, why) || !load_grid(dir, "c22.dat", N, c22, why) ||
            !load_grid(dir, "c33.dat", N, b, why) || !load_grid(dir, "rho.dat", N, r, why))
            return io_err(SEIDART_ERR_IO, why);
        double m = 0.0;
        for (size_t q = 0; q < N; ++q) m = fmax(m, fmax(a[q] / r[q], fmax(c22[q] / r[q], b[q] / r[q])));
        *dt = 0.7 * hmin / sqrt(3.0 * m);
    } else {
        const char* names[3] = {"e11.dat", "e22.dat", "e33.dat"};
        double emin = 1e300;
        for (const char* nm : names) {
            if (family == SEIDART_ELECTROMAG2 && strcmp(nm, "e22.dat") == 0) continue;
            if (!load_grid(dir, nm, N, a, why)) return io_err(SEIDART_ERR_IO, why);
            for (double v : a) emin = fmin(emin, v);
        }
        *dt = hmin / (2.0 * 2.9979458e8 / sqrt(emin));
    }
    return SEIDART_OK;
}

static int legacy_run(int family, int nx, int ny, int nz, double dx, double dy, double dz, int npml, const int* src,
                      int nstep, int single_output) {
    if (!src) return io_err(SEIDART_ERR_ARG, "src is NULL");
    SeidartDomain d{};
    const bool three = family == SEIDART_SEISMIC3 || family == SEIDART_ELECTROMAG3;
    d.dim = three ? 3.0 : (family == SEIDART_SEISMIC25 || family == SEIDART_ELECTROMAG25 ? 2.5 : 2.0);
    d.nx = nx; d.ny = three ? ny : 1; d.nz = nz;
    d.dx = dx; d.dy = dy; d.dz = dz; d.cpml = npml;
    SeidartSource s{};
    s.time_steps = nstep;
    s.xind = src[0];
    s.yind = three ? src[1] : 0;
    s.zind = three ? src[2] : src[1];
    const char* ky = getenv("KY");
    s.ky = ky ? atof(ky) : 0.0;
    const size_t N = (size_t)nx * (three ? ny : 1) * nz;
    double hmin = fmin(dx, dz);
    if (three) hmin = fmin(hmin, dy);
    int rc = legacy_dt(".", family, N, hmin, &s.dt);
    if (rc != SEIDART_OK) return rc;
    return seidart_run_files(".", family, SEIDART_FP64, &d, &s, SEIDART_DENSITY_ARITHMETIC, "ac", single_output, 1);
}

void seismic2_(int nx, int nz, double dx, double dz, int npoints_pml, int* src, int nstep, int single_output) {
    legacy_run(SEIDART_SEISMIC2, nx, 1, nz, dx, 1.0, dz, npoints_pml, src, nstep, single_output);
}
// The binding's seismic25 / electromag25 are 3D solvers on (nx, ny, nz) with
// 3D snapshots (legacy/cpmlfdtd_cbindings.f95:1088-1641, :2184-2640): they
// run the 3D loops, src = interior (xind, yind, zind).
void seismic25_(int nx, int ny, int nz, double dx, double dy, double dz, int npoints_pml, int* src, int nstep,
                int single_output) {
    legacy_run(SEIDART_SEISMIC3, nx, ny, nz, dx, dy, dz, npoints_pml, src, nstep, single_output);
}
void electromag2_(int nx, int nz, double dx, double dz, int npoints_pml, int* src, int nstep, int single_output) {
    legacy_run(SEIDART_ELECTROMAG2, nx, 1, nz, dx, 1.0, dz, npoints_pml, src, nstep, single_output);
}
void electromag25_(int nx, int ny, int nz, double dx, double dy, double dz, int npoints_pml, int* src, int nstep,
                   int single_output) {
    legacy_run(SEIDART_ELECTROMAG3, nx, ny, nz, dx, dy, dz, npoints_pml, src, nstep, single_output);
}
// The complex-valued legacy variants map onto the same (real) solvers.
void electromag2c_(int nx, int nz, double dx, double dz, int npoints_pml, int* src, int nstep, int single_output) {
    electromag2_(nx, nz, dx, dz, npoints_pml, src, nstep, single_output);
}
void electromag25c_(int nx, int ny, int nz, double dx, double dy, double dz, int npoints_pml, int* src, int nstep,
                    int single_output) {
    electromag25_(nx, ny, nz, dx, dy, dz, npoints_pml, src, nstep, single_output);
}

// ------------------------------------------------------------------- CLI
// seidartfdtd <input.json> [seismic=true|false] [density_method=...]
// (src/fortran/main.f08:31-119); extra flags precision=fp64|fp64fast|fp32 and
// snapshots=true|false are accepted, defaults keep the reference behaviour.
int seidart_cli_main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "Usage: seidartfdtd <input.json> [seismic=<true|false>] [density_method=<harmonic|geometric|arithmetic|none>]\n");
        return 1;
    }
    FILE* f = fopen(argv[1], "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", argv[1]); return 1; }
    std::string text;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    fclose(f);
    JsonReader js{text.c_str()};
    js.value("");
    if (!js.ok) { fprintf(stderr, "%s: malformed JSON\n", argv[1]); return 1; }
    bool seismic = true;
    std::string density = "arithmetic";  // main.f08:46
    int precision = SEIDART_FP64;
    bool snaps = true;
    for (int a = 2; a < argc; ++a) {
        std::string arg = argv[a];
        const size_t eq = arg.find('=');
        if (eq == std::string::npos) continue;
        const std::string k = trim(arg.substr(0, eq)), v = trim(arg.substr(eq + 1));
        if (k == "seismic") { if (v == "true") seismic = true; else if (v == "false") seismic = false; }
        else if (k == "density_method") density = v;
        else if (k == "precision")
            precision = v == "fp32" ? SEIDART_FP32 : v == "fp64fast" ? SEIDART_FP64_FAST : SEIDART_FP64;
        else if (k == "snapshots") snaps = v != "false";
    }
    int code = 0;
    if (density == "harmonic") code = 1;
    else if (density == "geometric") code = 2;
    else if (density == "arithmetic") code = 3;
    else if (density == "none") code = 4;
    else {
        fprintf(stderr, "Error: invalid density_method \"%s\".\n       Must be one of: harmonic, geometric, arithmetic, none\n", density.c_str());
        return 1;
    }
    SeidartDomain d{};
    double v;
    auto need = [&](const char* key, double& out) {
        if (!js.num(key, out)) { fprintf(stderr, "input.json: missing numeric %s\n", key); return false; }
        return true;
    };
    double nx, ny, nz, cp;
    if (!need("Domain.dim", d.dim) || !need("Domain.nx", nx) || !need("Domain.nz", nz) || !need("Domain.dx", d.dx) ||
        !need("Domain.dz", d.dz) || !need("Domain.cpml", cp))
        return 1;
    if (!js.num("Domain.ny", ny)) ny = 1;
    if (!js.num("Domain.dy", d.dy)) d.dy = 1.0;
    // main.f08:69-71: the solvers work on the padded grid
    d.cpml = (int)cp;
    d.nx = (int)nx + 2 * d.cpml;
    d.ny = (int)ny + 2 * d.cpml;
    d.nz = (int)nz + 2 * d.cpml;
    const std::string pre = seismic ? "Seismic.Source." : "Electromagnetic.Source.";
    SeidartSource s{};
    double ts, xi, yi, zi;
    if (!need((pre + "dt").c_str(), s.dt) || !need((pre + "time_steps").c_str(), ts) ||
        !need((pre + "xind").c_str(), xi) || !need((pre + "zind").c_str(), zi))
        return 1;
    if (!js.num(pre + "yind", yi)) yi = 0;
    s.time_steps = (int)ts; s.xind = (int)xi; s.yind = (int)yi; s.zind = (int)zi;
    const std::string stype = trim(js.text(pre + "source_type"));
    // plane-wave fields of the Source record (seidartio.f08:80-85, :101-106)
    SeidartPlaneWave pw{};
    {
        double v0;
        if (js.num(pre + "source_frequency", v0)) pw.frequency = v0;
        if (js.num(pre + "x-z_rotation", v0)) pw.x_z_rotation = v0;
        if (js.num(pre + "x-y_rotation", v0)) pw.x_y_rotation = v0;
        if (js.num(pre + "y-z_rotation", v0)) pw.y_z_rotation = v0;
        if (js.num(pre + "amplitude", v0)) pw.amplitude = v0;
        const std::string wl = trim(js.text(pre + "source_wavelet"));
        pw.wavelet = wl == "gaus1" ? 1 : wl == "gaus2" ? 2 : 0;  // wavelet(), plane_wave_source.f08:141-161
        pw.kind = SEIDART_PW_S;
    }
    const char* ky = getenv("KY");
    s.ky = ky ? atof(ky) : 0.0;
    // 2.5D solvers read SINGLE_OUTPUT and DENSITY_METHOD (default harmonic) from the environment
    // (cpmlfdtd.f08:689-716); 2D/3D write single precision (main.f08:93-116)
    int single = 1;
    int fam;
    if (d.dim == 3.0) {
        fam = seismic ? SEIDART_SEISMIC3 : SEIDART_ELECTROMAG3;  // main.f08:88-97
        printf(" Running 3D %s model with %d time steps\n", seismic ? "seismic" : "electromagnetic", s.time_steps);
    } else if (d.dim == 2.5) {
        fam = seismic ? SEIDART_SEISMIC25 : SEIDART_ELECTROMAG25;
        const char* so = getenv("SINGLE_OUTPUT");
        if (so) { std::string t = trim(so); single = !(t == "F" || t == "f" || t == ".false." || t == "false" || t == "0"); }
        if (seismic) {
            const char* dm = getenv("DENSITY_METHOD");
            std::string m = dm ? trim(dm) : std::string("harmonic");
            code = m == "geometric" ? 2 : m == "arithmetic" ? 3 : m == "none" ? 4 : 1;
        }
        printf(" Running 2.5D %s model with %d time steps\n", seismic ? "seismic" : "electromagnetic", s.time_steps);
    } else {
        fam = seismic ? SEIDART_SEISMIC2 : SEIDART_ELECTROMAG2;
        printf(" Running 2D %s model with %d time steps\n", seismic ? "seismic" : "electromagnetic", s.time_steps);
    }
    if (fam == SEIDART_ELECTROMAG2 || fam == SEIDART_ELECTROMAG25 || fam == SEIDART_SEISMIC2) d.ny = 1;
    (void)v;
    const int rc = seidart_run_files_pw(".", fam, precision, &d, &s, code, stype.empty() ? "ac" : stype.c_str(), single,
                                        snaps ? 1 : 0, &pw);
    if (rc == SEIDART_ERR_UNSTABLE) { fprintf(stderr, "code became unstable and blew up\n"); return 3; }
    if (rc != SEIDART_OK) { fprintf(stderr, "seidartfdtd: error %d: %s\n", rc, g_io_err.c_str()); return 4; }
    return 0;
}

}  // extern "C"
