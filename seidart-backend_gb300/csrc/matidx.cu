// matidx.cu -- material index of an FP32 3D model, built on the device.
//
// The staged stress kernel can read its 21 C_ij and 6 attenuation factors
// from a small table indexed by one byte per cell instead of 27 per-cell
// arrays.  That layout applies when the model holds at most S3_MAXMAT
// distinct coefficient tuples, as a model expanded from a material image
// does (one tuple per material).  The index is found here from the solver's
// own FP32 arrays, so the table holds exactly the values the per-cell layout
// would read:
//   1. matidx_hash: every cell hashes its 27 FP32 bit patterns; the lanes of
//      a warp with equal hashes elect one, which inserts the hash into a
//      64-slot open-addressing table (atomicCAS) and lowers the slot's
//      representative cell (atomicMin); a claimed slot is counted.
//   2. the host reads the table back, numbers the claimed slots by their
//      representative cell (a deterministic order) and uploads the numbers.
//   3. matidx_assign: every cell finds its slot, compares its 27 values with
//      the representative cell's bit for bit (a hash collision raises a flag
//      and the host keeps the per-cell layout) and writes its byte at its
//      place in the tile-packed layout ([tile][8][32], tile = tx + gx (ty + gy k)).
//   4. matidx_table: the representative cells' values form the table.
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "kernels.h"

namespace {

constexpr int NSLOT = 64;

struct HashTable {
    unsigned long long key[NSLOT];  // 0 = empty
    unsigned long long rep[NSLOT];  // smallest cell holding the tuple
    int count;                      // claimed slots
    int collision;                  // a cell's tuple differs from its slot's representative
    int slot_id[NSLOT];             // material number of each claimed slot (set by the host)
};

__device__ __forceinline__ float coef(const S3Args<float>& A, int q, size_t c) {
    return q < 21 ? A.C[q][c] : A.g[q - 21][c];
}

__device__ __forceinline__ unsigned long long tuple_hash(const S3Args<float>& A, size_t c) {
    // 64-bit FNV-1a over the 27 bit patterns, then a final avalanche
    unsigned long long h = 1469598103934665603ull;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
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

__global__ void matidx_hash(S3Args<float> A, size_t ncell, HashTable* T) {
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

__global__ void matidx_assign(S3Args<float> A, int nx, int ny, int nz, HashTable* T, unsigned char* ids) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, k = blockIdx.z;
    const size_t t = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * k);
    unsigned char* dst = ids + t * 256 + threadIdx.y * 32 + threadIdx.x;
    if (x >= nx || y >= ny) {
        *dst = 0;  // outside the grid: any material (the kernels do not update these slots)
        return;
    }
    const size_t c = (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * k);
    const int s = find_slot(T, tuple_hash(A, c));
    if (s < 0) {
        atomicExch(&T->collision, 1);
        *dst = 0;
        return;
    }
    const size_t r = (size_t)T->rep[s];
    bool same = true;
#pragma unroll
    for (int q = 0; q < 27; ++q) same = same && __float_as_uint(coef(A, q, c)) == __float_as_uint(coef(A, q, r));
    if (!same) atomicExch(&T->collision, 1);
    *dst = (unsigned char)T->slot_id[s];
}

__global__ void matidx_table(S3Args<float> A, const HashTable* T, float* tab) {
    const int s = blockIdx.x, q = threadIdx.x;
    if (q >= 27 || T->key[s] == 0ull) return;
    tab[T->slot_id[s] * 27 + q] = coef(A, q, (size_t)T->rep[s]);
}

}  // namespace

int seismic3_material_index(const S3Args<float>& a, int nx, int ny, int nz, unsigned char** ids_out, float** tab_out,
                            int* nmat_out, cudaStream_t st) {
    *ids_out = nullptr;
    *tab_out = nullptr;
    *nmat_out = 0;
    const size_t ncell = (size_t)nx * ny * nz;
    const int gx = (nx + 31) / 32, gy = (ny + 7) / 8;
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
    matidx_hash<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(a, ncell, T);
    HashTable h{};
    if (cudaMemcpyAsync(&h, T, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(true);
    if (h.count < 1 || h.count > S3_MAXMAT) return fail(false);
    // number the tuples by their first cell
    std::vector<std::pair<unsigned long long, int>> order;
    for (int s = 0; s < NSLOT; ++s)
        if (h.key[s]) order.push_back({h.rep[s], s});
    std::sort(order.begin(), order.end());
    for (int s = 0; s < NSLOT; ++s) h.slot_id[s] = 0;
    for (size_t m = 0; m < order.size(); ++m) h.slot_id[order[m].second] = (int)m;
    const size_t nbytes = (size_t)gx * gy * nz * 256;
    int* dev_slot_id = (int*)((char*)T + offsetof(HashTable, slot_id));
    int* dev_collision = (int*)((char*)T + offsetof(HashTable, collision));
    if (cudaMemcpyAsync(dev_slot_id, h.slot_id, sizeof h.slot_id, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMalloc((void**)&ids, nbytes) != cudaSuccess ||
        cudaMalloc((void**)&tab, sizeof(float) * S3_MAXMAT * 27) != cudaSuccess ||
        cudaMemsetAsync(tab, 0, sizeof(float) * S3_MAXMAT * 27, st) != cudaSuccess)
        return fail(true);
    matidx_assign<<<dim3(gx, gy, nz), dim3(32, 8), 0, st>>>(a, nx, ny, nz, T, ids);
    matidx_table<<<NSLOT, 32, 0, st>>>(a, T, tab);
    int collision = 0;
    if (cudaMemcpyAsync(&collision, dev_collision, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(true);
    if (collision) return fail(false);
    cudaFree(T);
    *ids_out = ids;
    *tab_out = tab;
    *nmat_out = (int)order.size();
    return (int)order.size();
}
