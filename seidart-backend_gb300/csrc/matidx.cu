// matidx.cu -- material index of an FP32 elastic model, built on the device.
//
// The 3D staged stress kernel can read its 21 C_ij and 6 attenuation
// factors, and the 2D batch walk its 9 stress coefficients, from a small
// table indexed by one byte per cell instead of per-cell arrays.  That
// layout applies when the model holds at most S3_MAXMAT distinct coefficient
// tuples, as a model expanded from a material image does (one tuple per
// material).  The index is found here from the solver's own FP32 arrays, so
// the table holds exactly the values the per-cell layout would read:
//   1. matidx_hash: every cell hashes its 27 FP32 bit patterns; the lanes of
//      a warp with equal hashes elect one, which inserts the hash into a
//      128-slot open-addressing table (atomicCAS) and lowers the slot's
//      representative cell (atomicMin); a claimed slot is counted.
//   2. the host reads the table back, numbers the claimed slots by their
//      representative cell (a deterministic order) and uploads the numbers.
//   3. matidx_assign: every cell finds its slot, compares its 27 values with
//      the representative cell's bit for bit (a hash collision raises a flag
//      and the host keeps the per-cell layout) and writes its byte: in 3D at
//      its place in the tile-packed layout ([tile][8][32], tile = tx + gx
//      (ty + gy k)), in 2D in grid order.
//   4. matidx_table: the representative cells' values form the table.
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "kernels.h"

namespace {

constexpr int NSLOT = 128;

struct HashTable {
    unsigned long long key[NSLOT];  // 0 = empty
    unsigned long long rep[NSLOT];  // smallest cell holding the tuple
    int count;                      // claimed slots
    int collision;                  // a cell's tuple differs from its slot's representative
    int slot_id[NSLOT];             // tuple number of each claimed slot (set by the host)
};

// the coefficient arrays of one model (27 for seismic3, 9 for seismic2)
struct Arr {
    const float* p[27];
    int n;
};

__device__ __forceinline__ float coef(const Arr& A, int q, size_t c) { return A.p[q][c]; }

__device__ __forceinline__ unsigned long long tuple_hash(const Arr& A, size_t c) {
    // 64-bit FNV-1a over the bit patterns, then a final avalanche
    unsigned long long h = 1469598103934665603ull;
    for (int q = 0; q < A.n; ++q) {
        h ^= (unsigned long long)__float_as_uint(coef(A, q, c));
        h *= 1099511628211ull;
    }
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    return h ? h : 1ull;
}

__device__ __forceinline__ int find_slot(const HashTable* T, unsigned long long h) {
    int s = (int)(h % NSLOT);
    for (int n = 0; n < NSLOT; ++n, s = (s + 1) % NSLOT)
        if (T->key[s] == h) return s;
    return -1;
}

__global__ void matidx_hash(Arr A, size_t ncell, HashTable* T) {
    const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const bool in = c < ncell;
    const unsigned long long h = in ? tuple_hash(A, c) : 0ull;
    const unsigned lanes = __match_any_sync(0xffffffffu, h);
    const int lane = threadIdx.x & 31;
    if (!in || lane != __ffs(lanes) - 1) return;  // one lane per distinct hash of the warp
    int s = (int)(h % NSLOT);
    for (int n = 0; n < NSLOT; ++n, s = (s + 1) % NSLOT) {
        const unsigned long long prev = atomicCAS(&T->key[s], 0ull, h);
        if (prev == 0ull) atomicAdd(&T->count, 1);
        if (prev == 0ull || prev == h) {
            atomicMin(&T->rep[s], (unsigned long long)c);
            return;
        }
    }
    atomicAdd(&T->count, NSLOT + 1);  // table full: far more tuples than the layout takes
}

// the byte of cell c: its slot's number, after a bit-for-bit check against
// the slot's representative cell
__device__ __forceinline__ unsigned char assign_cell(const Arr& A, HashTable* T, size_t c) {
    const int s = find_slot(T, tuple_hash(A, c));
    if (s < 0) {
        atomicExch(&T->collision, 1);
        return 0;
    }
    const size_t r = (size_t)T->rep[s];
    bool same = true;
    for (int q = 0; q < A.n; ++q) same = same && __float_as_uint(coef(A, q, c)) == __float_as_uint(coef(A, q, r));
    if (!same) atomicExch(&T->collision, 1);
    return (unsigned char)T->slot_id[s];
}

// 3D: the bytes tile-packed as the staged stress kernel copies them
__global__ void matidx_assign_tiled(Arr A, int nx, int ny, int nz, HashTable* T, unsigned char* ids) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, k = blockIdx.z;
    const size_t t = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * k);
    unsigned char* dst = ids + t * 256 + threadIdx.y * 32 + threadIdx.x;
    if (x >= nx || y >= ny) {
        *dst = 0;  // outside the grid: any material (the kernels do not update these slots)
        return;
    }
    *dst = assign_cell(A, T, (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * k));
}

// 2D and others: one byte per cell in the grid's own order
__global__ void matidx_assign_linear(Arr A, size_t ncell, HashTable* T, unsigned char* ids) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x)
        ids[c] = assign_cell(A, T, c);
}

__global__ void matidx_table(Arr A, const HashTable* T, float* tab) {
    const int s = blockIdx.x, q = threadIdx.x;
    if (q >= A.n || T->key[s] == 0ull) return;
    tab[T->slot_id[s] * A.n + q] = coef(A, q, (size_t)T->rep[s]);
}

}  // namespace

namespace {

// Hash, number, assign and tabulate (steps 1-4 above).  tiled: the 3D
// tile-packed byte layout on an nx x ny x nz grid; else one byte per cell in
// grid order.  Returns the number of materials, 0 when they are more than
// max_tuples (or on an allocation failure).
int build_index(const Arr& A, size_t ncell, bool tiled, int nx, int ny, int nz, unsigned char** ids_out,
                float** tab_out, cudaStream_t st, int max_tuples = S3_MAXMAT) {
    *ids_out = nullptr;
    *tab_out = nullptr;
    HashTable* T = nullptr;
    unsigned char* ids = nullptr;
    float* tab = nullptr;
    auto fail = [&](bool cuda_error) {
        if (cuda_error) cudaGetLastError();
        if (T) cudaFree(T);
        if (ids) cudaFree(ids);
        if (tab) cudaFree(tab);
        return 0;
    };
    if (cudaMalloc((void**)&T, sizeof(HashTable)) != cudaSuccess) return fail(true);
    HashTable h0{};
    for (int s = 0; s < NSLOT; ++s) h0.rep[s] = ~0ull;
    if (cudaMemcpyAsync(T, &h0, sizeof h0, cudaMemcpyHostToDevice, st) != cudaSuccess) return fail(true);
    matidx_hash<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(A, ncell, T);
    HashTable h{};
    if (cudaMemcpyAsync(&h, T, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(true);
    if (h.count < 1 || h.count > max_tuples) return fail(false);
    // number the tuples by their first cell
    std::vector<std::pair<unsigned long long, int>> order;
    for (int s = 0; s < NSLOT; ++s)
        if (h.key[s]) order.push_back({h.rep[s], s});
    std::sort(order.begin(), order.end());
    for (int s = 0; s < NSLOT; ++s) h.slot_id[s] = 0;
    for (size_t m = 0; m < order.size(); ++m) h.slot_id[order[m].second] = (int)m;
    const int gx = (nx + 31) / 32, gy = (ny + 7) / 8;
    const size_t nbytes = tiled ? (size_t)gx * gy * nz * 256 : ncell;
    int* dev_slot_id = (int*)((char*)T + offsetof(HashTable, slot_id));
    int* dev_collision = (int*)((char*)T + offsetof(HashTable, collision));
    if (cudaMemcpyAsync(dev_slot_id, h.slot_id, sizeof h.slot_id, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMalloc((void**)&ids, nbytes) != cudaSuccess ||
        cudaMalloc((void**)&tab, sizeof(float) * max_tuples * A.n) != cudaSuccess ||
        cudaMemsetAsync(tab, 0, sizeof(float) * max_tuples * A.n, st) != cudaSuccess)
        return fail(true);
    if (tiled) matidx_assign_tiled<<<dim3(gx, gy, nz), dim3(32, 8), 0, st>>>(A, nx, ny, nz, T, ids);
    else matidx_assign_linear<<<4 * 152, 256, 0, st>>>(A, ncell, T, ids);
    matidx_table<<<NSLOT, 32, 0, st>>>(A, T, tab);
    int collision = 0;
    if (cudaMemcpyAsync(&collision, dev_collision, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(true);
    if (collision) return fail(false);
    cudaFree(T);
    *ids_out = ids;
    *tab_out = tab;
    return (int)order.size();
}

}  // namespace

int seismic3_material_index(const S3Args<float>& a, int nx, int ny, int nz, unsigned char** ids_out, float** tab_out,
                            int* nmat_out, cudaStream_t st) {
    Arr A{};
    for (int q = 0; q < 21; ++q) A.p[q] = a.C[q];
    for (int q = 0; q < 6; ++q) A.p[21 + q] = a.g[q];
    A.n = 27;
    *nmat_out = build_index(A, (size_t)nx * ny * nz, true, nx, ny, nz, ids_out, tab_out, st);
    return *nmat_out;
}

int seismic2_material_index(const float* const* coef, size_t ncell, unsigned char** ids_out, float** tab_out,
                            int* nmat_out, cudaStream_t st) {
    Arr A{};
    for (int q = 0; q < 9; ++q) A.p[q] = coef[q];
    A.n = 9;
    *nmat_out = build_index(A, ncell, false, 0, 0, 0, ids_out, tab_out, st);
    return *nmat_out;
}

int seismic3_cpml_index(const S3Args<float>& a, int nx, int ny, int nz, unsigned char** ids_out, float** tab_out,
                        int* ntup_out, cudaStream_t st) {
    Arr A{};
    for (int q = 0; q < 6; ++q) A.p[q] = a.cpml[q];
    A.n = 6;
    *ntup_out = build_index(A, (size_t)nx * ny * nz, true, nx, ny, nz, ids_out, tab_out, st, S3_MAXCPML);
    return *ntup_out;
}
