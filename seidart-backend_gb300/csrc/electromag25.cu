// electromag25.cu -- 2.5D anisotropic E/H CPML-FDTD on complex fields with a
// full 3x3 permittivity inverse and conductivity tensor,
// src/fortran/cpmlfdtd.f08:3095-3331.
//
//   e25_h : Hx (:3106-3119), Hy (:3132-3151), Hz (:3164-3177), 4th order.
//   e25_e : E from curl H and sigma E (:3195-3245), point source
//           (:3261-3266), Dirichlet ring on E (:3270-3283), max-norm (:3308).
// The H loops never write the outer ring, so the reference's H ring zeroing
// (:3285-3298) only keeps it at zero; e25_h writes zero there each step.
// E_old equals E at the start of every E update, so it is not stored.
#include "common.cuh"
#include "kernels.h"

namespace {
constexpr int BX = 32, BY = 8;

struct cx {
    real re, im;
};
__device__ __forceinline__ cx ld(const real* a, size_t c) {
#if !SD_F32
    const double2 v = reinterpret_cast<const double2*>(a)[c];
#else
    const float2 v = reinterpret_cast<const float2*>(a)[c];
#endif
    return cx{v.x, v.y};
}
__device__ __forceinline__ void stc(real* a, size_t c, cx z) {
#if !SD_F32
    reinterpret_cast<double2*>(a)[c] = make_double2(z.re, z.im);
#else
    reinterpret_cast<float2*>(a)[c] = make_float2(z.re, z.im);
#endif
}
__device__ __forceinline__ cx operator+(cx a, cx b) { return cx{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cx operator-(cx a, cx b) { return cx{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cx operator*(real r, cx a) { return cx{r * a.re, r * a.im}; }
__device__ __forceinline__ cx operator*(cx a, real r) { return cx{a.re * r, a.im * r}; }
__device__ __forceinline__ cx cdiv(cx a, real r) {
#if SD_EXACT
    return cx{a.re / r, a.im / r};
#else
    return cx{a.re * r, a.im * r};
#endif
}
__device__ __forceinline__ cx iky(real ky, cx a) { return cx{-(ky * a.im), ky * a.re}; }

#define IX(fi, fk) ((size_t)((fi) - 1) + (size_t)nx * (size_t)((fk) - 1))

__device__ __forceinline__ cx d4(const real* f, size_t p1, size_t p0, size_t p2, size_t m1, real h) {
    return cdiv((real)27 * (ld(f, p1) - ld(f, p0)) - (ld(f, p2) - ld(f, m1)), h);
}
__device__ __forceinline__ cx cpml(real* m, size_t c, real b, real aa, real k, cx d) {
    const cx mv = b * ld(m, c) + aa * d;
    stc(m, c, mv);
    return cdiv(d, k) + mv;
}

__global__ void __launch_bounds__(BX* BY) e25_h(E25Args<real> a) {
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int k = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    if (i > nx || k > nz) return;
    const size_t c = IX(i, k);
    if (i == 1 || i == nx || k == 1 || k == nz) {
        stc(a.f[3], c, cx{0, 0}); stc(a.f[4], c, cx{0, 0}); stc(a.f[5], c, cx{0, 0});
        return;
    }
    const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && k - 1 >= a.box.k0 && k - 1 < a.box.k1);
    const real *Ex = a.f[0], *Ey = a.f[1], *Ez = a.f[2];
    const real *kaph = a.cpml[1], *ach = a.cpml[3], *bch = a.cpml[5];
#if SD_EXACT
    const real hx = 24.0 * a.dx, hz = 24.0 * a.dz;
#else
    const real hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
#endif
    const real dtmu = a.dtmu, ky = a.ky;
    if (k >= 2 && k <= nz - 2 && i >= 2 && i <= nx - 1) {
        cx dEy_dz = d4(Ey, IX(i, k + 1), c, IX(i, k + 2), IX(i, k - 1), hz);
        if (pml) dEy_dz = cpml(a.mem[1], c, bch[c], ach[c], kaph[c], dEy_dz);
        stc(a.f[3], c, ld(a.f[3], c) - dtmu * (iky(ky, ld(Ez, c)) - dEy_dz));
    }
    if (k >= 2 && k <= nz - 2 && i >= 2 && i <= nx - 2) {
        cx dEx_dz = d4(Ex, IX(i, k + 1), c, IX(i, k + 2), IX(i, k - 1), hz);
        cx dEz_dx = d4(Ez, IX(i + 1, k), c, IX(i + 2, k), IX(i - 1, k), hx);
        if (pml) {
            dEx_dz = cpml(a.mem[2], c, bch[c], ach[c], kaph[c], dEx_dz);
            dEz_dx = cpml(a.mem[3], c, bch[c], ach[c], kaph[c], dEz_dx);
        }
        stc(a.f[4], c, ld(a.f[4], c) - dtmu * (dEx_dz - dEz_dx));
    }
    if (k >= 2 && k <= nz - 1 && i >= 2 && i <= nx - 2) {
        cx dEy_dx = d4(Ey, IX(i + 1, k), c, IX(i + 2, k), IX(i - 1, k), hx);
        if (pml) dEy_dx = cpml(a.mem[0], c, bch[c], ach[c], kaph[c], dEy_dx);
        stc(a.f[5], c, ld(a.f[5], c) - dtmu * (dEy_dx - iky(ky, ld(Ex, c))));
    }
}

__global__ void __launch_bounds__(BX* BY) e25_e(E25Args<real> a, StepInfo si) {
    const int it = *si.step;
    __shared__ double red[BX * BY / 32];
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int k = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    double nrm = 0.0;
    float sq = 0.f, w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // FP32 build: squared norm and components
    if (i <= nx && k <= nz) {
        const size_t c = IX(i, k);
        cx ex = ld(a.f[0], c), ey = ld(a.f[1], c), ez = ld(a.f[2], c);
        if (k >= 3 && k <= nz - 2 && i >= 3 && i <= nx - 2) {
            const real *Hx = a.f[3], *Hy = a.f[4], *Hz = a.f[5];
#if SD_EXACT
            const real hx = 24.0 * a.dx, hz = 24.0 * a.dz;
#else
            const real hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
#endif
            const cx dHz_dy = iky(a.ky, ld(Hz, c));
            cx dHy_dz = d4(Hy, c, IX(i, k - 1), IX(i, k + 1), IX(i, k - 2), hz);
            cx dHx_dz = d4(Hx, c, IX(i, k - 1), IX(i, k + 1), IX(i, k - 2), hz);
            cx dHz_dx = d4(Hz, c, IX(i - 1, k), IX(i + 1, k), IX(i - 2, k), hx);
            cx dHy_dx = d4(Hy, c, IX(i - 1, k), IX(i + 1, k), IX(i - 2, k), hx);
            const cx dHx_dy = iky(a.ky, ld(Hx, c));
            const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && k - 1 >= a.box.k0 && k - 1 < a.box.k1);
            if (pml) {
                const real b = a.cpml[4][c], aa = a.cpml[2][c], kk = a.cpml[0][c];
                dHy_dz = cpml(a.mem[6], c, b, aa, kk, dHy_dz);
                dHx_dz = cpml(a.mem[5], c, b, aa, kk, dHx_dz);
                dHz_dx = cpml(a.mem[4], c, b, aa, kk, dHz_dx);
                dHy_dx = cpml(a.mem[7], c, b, aa, kk, dHy_dx);
            }
            const real s11 = a.sig[0][c], s12 = a.sig[1][c], s13 = a.sig[2][c], s22 = a.sig[3][c],
                       s23 = a.sig[4][c], s33 = a.sig[5][c];
            const cx rx = (dHz_dy - dHy_dz) - (s11 * ex + s12 * ey + s13 * ez);
            const cx ry = (dHx_dz - dHz_dx) - (s12 * ex + s22 * ey + s23 * ez);
            const cx rz = (dHy_dx - dHx_dy) - (s13 * ex + s23 * ey + s33 * ez);
            const real dt = a.dt;
            const cx nx_ = ex + (a.inv[0][c] * rx + a.inv[1][c] * ry + a.inv[2][c] * rz) * dt;
            const cx ny_ = ey + (a.inv[3][c] * rx + a.inv[4][c] * ry + a.inv[5][c] * rz) * dt;
            const cx nz_ = ez + (a.inv[6][c] * rx + a.inv[7][c] * ry + a.inv[8][c] * rz) * dt;
            ex = nx_; ey = ny_; ez = nz_;
        }
        if (i - 1 == a.isrc && k - 1 == a.ksrc) {
            // cpmlfdtd.f08:3261-3266: srcx*dt/eps11 on the real part
            if (a.src[0]) ex.re = ex.re + (real)a.src[0][it - 1] * a.dt / a.eabs[0][c];
            if (a.src[1]) ey.re = ey.re + (real)a.src[1][it - 1] * a.dt / a.eabs[1][c];
            if (a.src[2]) ez.re = ez.re + (real)a.src[2][it - 1] * a.dt / a.eabs[2][c];
        }
        if (i == 1 || i == nx || k == 1 || k == nz) { ex = cx{0, 0}; ey = cx{0, 0}; ez = cx{0, 0}; }
        stc(a.f[0], c, ex);
        stc(a.f[1], c, ey);
        stc(a.f[2], c, ez);
#if !SD_F32
        const double n1 = (double)ex.re * ex.re + (double)ex.im * ex.im;
        const double n2 = (double)ey.re * ey.re + (double)ey.im * ey.im;
        const double n3 = (double)ez.re * ez.re + (double)ez.im * ez.im;
        nrm = sqrt(n1 + n2 + n3);
#else
        sq = (ex.re * ex.re + ex.im * ex.im) + (ey.re * ey.re + ey.im * ey.im) + (ez.re * ez.re + ez.im * ez.im);
        w[0] = ex.re; w[1] = ex.im; w[2] = ey.re; w[3] = ey.im; w[4] = ez.re; w[5] = ez.im;
#endif
    }
#if !SD_F32
    nrm = block_max<BX * BY / 32>(nrm, red);
#else
    __shared__ float redf[BX * BY / 32];
    nrm = block_norm_f32<BX * BY / 32>(sq, [&] { return sqrt((double)w[0] * w[0] + (double)w[1] * w[1] + ((double)w[2] * w[2] + (double)w[3] * w[3]) +
                                                       ((double)w[4] * w[4] + (double)w[5] * w[5])); }, redf, red);
#endif
    if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(&a.norms[it - 1], nrm);
}

// Receiver gather (after the Dirichlet ring, like the reference's per-step
// snapshot) and advance of the device step counter; always the last
// kernel of a step.
__global__ void e25_epilogue(E25Args<real> a, StepInfo s) {
    const int it = *s.step;
    for (int r = threadIdx.x; r < s.nrec; r += blockDim.x) {
        const size_t base = (size_t)(it - 1) * 3 * s.nrec;
    #pragma unroll
        for (int q = 0; q < 3; ++q) {
            const cx v = ld(a.f[q], (size_t)s.rec[r]);
            a.traces[2 * (base + (size_t)q * s.nrec + r)] = v.re;
            a.traces[2 * (base + (size_t)q * s.nrec + r) + 1] = v.im;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *s.step = it + 1;
}
}  // namespace

void SD_NAME(launch_electromag25)(const E25Args<real>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h) {
    const dim3 blk(BX, BY), grd((a.nx + BX - 1) / BX, (a.nz + BY - 1) / BY);
    e25_h<<<grd, blk, 0, st>>>(a);
    if (h) h->fn(h->ctx, 0, "e25_h");
    e25_e<<<grd, blk, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 1, "e25_e");
    e25_epilogue<<<1, 256, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 2, "e25_epilogue");
}
