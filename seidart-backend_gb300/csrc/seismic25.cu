// seismic25.cu -- 2.5D anisotropic elastic CPML-FDTD on complex fields
// (d/dy -> i*ky), src/fortran/cpmlfdtd.f08:931-1313.
//
//   s25_stress   : the four stress loops (:941-1117) fused into one pass;
//                  each cell evaluates the loops whose bounds contain it.
//   s25_velocity : vx, vy, vz (:1130-1202), force source (:1274-1276),
//                  Dirichlet ring (:1280-1285), max-norm (:1291).
// Mixed real/complex arithmetic is component-wise: real*complex scales both
// parts, complex/real divides both, complex+real touches only the real part,
// and (0,1)*ky*z = (-(ky*Im z), ky*Re z).
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
__device__ __forceinline__ cx operator-(cx a) { return cx{-a.re, -a.im}; }
__device__ __forceinline__ cx cdiv(cx a, real r) {
#if SD_EXACT
    return cx{a.re / r, a.im / r};
#else
    return cx{a.re * r, a.im * r};  // FP32: r already holds the reciprocal
#endif
}
__device__ __forceinline__ cx iky(real ky, cx a) { return cx{-(ky * a.im), ky * a.re}; }

#define IX(fi, fk) ((size_t)((fi) - 1) + (size_t)nx * (size_t)((fk) - 1))

// (27(f[p1]-f[p0]) - (f[p2]-f[m1])) / (24 h)   [FP32: h is 1/(24 h)]
__device__ __forceinline__ cx d4(const real* f, size_t p1, size_t p0, size_t p2, size_t m1, real h) {
    return cdiv((real)27 * (ld(f, p1) - ld(f, p0)) - (ld(f, p2) - ld(f, m1)), h);
}
// m = b m + a d ; return d/k + m
__device__ __forceinline__ cx cpml(real* m, size_t c, real b, real aa, real k, cx d) {
    const cx mv = b * ld(m, c) + aa * d;
    stc(m, c, mv);
    return cdiv(d, k) + mv;
}

template <int L>
__device__ __forceinline__ void stress_loop(const S25Args<real>& a, int i, int k, size_t c, bool pml) {
    const int nx = a.nx;
    constexpr bool xfwd = (L == 1 || L == 4), zfwd = (L >= 3);
    constexpr bool xhalf = (L == 1 || L == 4), zhalf = (L != 1);
#if SD_EXACT
    const real hx = 24.0 * a.dx, hz = 24.0 * a.dz;
#else
    const real hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
#endif
    cx gx[3], gy[3], gz[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const real* v = a.f[q];
        gx[q] = xfwd ? d4(v, IX(i + 1, k), c, IX(i + 2, k), IX(i - 1, k), hx)
                     : d4(v, c, IX(i - 1, k), IX(i + 1, k), IX(i - 2, k), hx);
        gy[q] = iky(a.ky, ld(v, c));
        gz[q] = zfwd ? d4(v, IX(i, k + 1), c, IX(i, k + 2), IX(i, k - 1), hz)
                     : d4(v, c, IX(i, k - 1), IX(i, k + 1), IX(i, k - 2), hz);
    }
    if (pml) {
        const real bx = a.cpml[xhalf ? 5 : 4][c], ax = a.cpml[xhalf ? 3 : 2][c], kx = a.cpml[xhalf ? 1 : 0][c];
        const real bz = a.cpml[zhalf ? 5 : 4][c], az = a.cpml[zhalf ? 3 : 2][c], kz = a.cpml[zhalf ? 1 : 0][c];
#pragma unroll
        for (int q = 0; q < 3; ++q) gx[q] = cpml(a.mem[6 * (L - 1) + q], c, bx, ax, kx, gx[q]);
#pragma unroll
        for (int q = 0; q < 3; ++q) gz[q] = cpml(a.mem[6 * (L - 1) + 3 + q], c, bz, az, kz, gz[q]);
    }
    const cx e4 = gz[1] + gy[2], e5 = gz[0] + gx[2], e6 = gx[1] + gy[0];
    const real dt = a.dt;
    auto upd = [&](real* s, int c1, int c2, int c3, int c4, int c5, int c6, const real* g) {
        const cx acc = a.C[c1][c] * gx[0] + a.C[c2][c] * gy[1] + a.C[c3][c] * gz[2] + a.C[c4][c] * e4 +
                       a.C[c5][c] * e5 + a.C[c6][c] * e6;
#if SD_EXACT
        stc(s, c, cdiv(ld(s, c) + acc * dt, 1.0 + g[c] * dt));
#else
        stc(s, c, (ld(s, c) + acc * dt) * g[c]);
#endif
    };
    // C index: 0 c11 1 c12 2 c13 3 c14 4 c15 5 c16 6 c22 7 c23 8 c24 9 c25 10 c26
    //          11 c33 12 c34 13 c35 14 c36 15 c44 16 c45 17 c46 18 c55 19 c56 20 c66
    if (L == 1) {
        upd(a.f[3], 0, 1, 2, 3, 4, 5, a.g[0]);       // sigmaxx, gamma_x
        upd(a.f[6], 1, 6, 7, 8, 9, 10, a.g[1]);      // sigmayy, gamma_y
        upd(a.f[8], 2, 7, 11, 12, 13, 14, a.g[2]);   // sigmazz, gamma_z
    } else if (L == 2) {
        upd(a.f[4], 5, 10, 14, 17, 19, 20, a.g[3]);  // sigmaxy, gamma_xy
    } else if (L == 3) {
        upd(a.f[5], 4, 9, 13, 16, 18, 19, a.g[5]);   // sigmaxz, gamma_xz
    } else {
        upd(a.f[7], 3, 8, 12, 15, 16, 17, a.g[4]);   // sigmayz, gamma_yz
    }
}

__global__ void __launch_bounds__(BX* BY) s25_stress(S25Args<real> a) {
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int k = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    if (i > nx || k > nz) return;
    const size_t c = IX(i, k);
    const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && k - 1 >= a.box.k0 && k - 1 < a.box.k1);
    if (k >= 3 && k <= nz - 1 && i >= 2 && i <= nx - 2) stress_loop<1>(a, i, k, c, pml);
    if (k >= 3 && k <= nz - 1 && i >= 3 && i <= nx - 1) stress_loop<2>(a, i, k, c, pml);
    if (k >= 2 && k <= nz - 2 && i >= 3 && i <= nx - 1) stress_loop<3>(a, i, k, c, pml);
    if (k >= 2 && k <= nz - 2 && i >= 2 && i <= nx - 2) stress_loop<4>(a, i, k, c, pml);
}

__global__ void __launch_bounds__(BX* BY) s25_velocity(S25Args<real> a, StepInfo si) {
    const int it = *si.step;
    __shared__ double red[BX * BY / 32];
    const int i = blockIdx.x * BX + threadIdx.x + 1;
    const int k = blockIdx.y * BY + threadIdx.y + 1;
    const int nx = a.nx, nz = a.nz;
    double nrm = 0.0;
    float sq = 0.f, w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // FP32 build: squared norm and components
    if (i <= nx && k <= nz) {
        const size_t c = IX(i, k);
        const bool pml = !(i - 1 >= a.box.i0 && i - 1 < a.box.i1 && k - 1 >= a.box.k0 && k - 1 < a.box.k1);
        const real *sxx = a.f[3], *sxy = a.f[4], *sxz = a.f[5], *syy = a.f[6], *syz = a.f[7], *szz = a.f[8];
        const real dt = a.dt, ky = a.ky;
#if SD_EXACT
        const real hx = 24.0 * a.dx, hz = 24.0 * a.dz;
#else
        const real hx = 1.0f / (24.0f * a.dx), hz = 1.0f / (24.0f * a.dz);
#endif
        const real *kap = a.cpml[0], *kaph = a.cpml[1], *ac = a.cpml[2], *ach = a.cpml[3], *bc = a.cpml[4],
                   *bch = a.cpml[5];
        cx vx = ld(a.f[0], c), vy = ld(a.f[1], c), vz = ld(a.f[2], c);
        if (k >= 3 && k <= nz - 1 && i >= 3 && i <= nx - 1) {
            cx d1 = cdiv((real)27 * ld(sxx, c) - (real)27 * ld(sxx, IX(i - 1, k)) + ld(sxx, IX(i - 2, k)), hx);
            cx d2 = iky(ky, ld(sxy, c));
            cx d3 = cdiv((real)27 * ld(sxz, c) - (real)27 * ld(sxz, IX(i, k - 1)) + ld(sxz, IX(i, k - 2)), hz);
            if (pml) {
                d1 = cpml(a.mem[24], c, bch[c], ach[c], kaph[c], d1);
                d3 = cpml(a.mem[25], c, bch[c], ach[c], kaph[c], d3);
            }
            vx = vx + (cdiv(d1, a.rho9[0][c]) + cdiv(d2, a.rho9[1][c]) + cdiv(d3, a.rho9[2][c])) * dt;
        }
        if (k >= 3 && k <= nz - 1 && i >= 2 && i <= nx - 2) {
            cx d1 = cdiv(-((real)27 * ld(sxy, c)) + (real)27 * ld(sxy, IX(i + 1, k)) - ld(sxy, IX(i + 2, k)), hx);
            cx d2 = iky(ky, ld(syy, c));
            cx d3 = cdiv((real)27 * ld(syz, c) - (real)27 * ld(syz, IX(i, k - 1)) + ld(syz, IX(i, k - 2)), hz);
            if (pml) {
                d1 = cpml(a.mem[26], c, bch[c], ach[c], kaph[c], d1);
                d3 = cpml(a.mem[27], c, bc[c], ac[c], kap[c], d3);
            }
            vy = vy + (cdiv(d1, a.rho9[3][c]) + cdiv(d2, a.rho9[4][c]) + cdiv(d3, a.rho9[5][c])) * dt;
        }
        if (k >= 2 && k <= nz - 2 && i >= 2 && i <= nx - 2) {
            cx d1 = cdiv(-((real)27 * ld(sxz, c)) + (real)27 * ld(sxz, IX(i + 1, k)) - ld(sxz, IX(i + 2, k)), hx);
            cx d2 = iky(ky, ld(syz, c));
            cx d3 = cdiv(-((real)27 * ld(szz, c)) + (real)27 * ld(szz, IX(i, k + 1)) - ld(szz, IX(i, k + 2)), hz);
            if (pml) {
                d1 = cpml(a.mem[28], c, bch[c], ach[c], kaph[c], d1);
                d3 = cpml(a.mem[29], c, bch[c], ach[c], kaph[c], d3);
            }
            vz = vz + (cdiv(d1, a.rho9[6][c]) + cdiv(d2, a.rho9[7][c]) + cdiv(d3, a.rho9[8][c])) * dt;
        }
        // force source, cpmlfdtd.f08:1274-1276 (real part, with dt)
        const int is = a.isrc + 1, ks = a.ksrc + 1;
        if (a.src[0] && i == is + 1 && k == ks) vx.re = vx.re + cdiv(cx{(real)a.src[0][it - 1] * dt, 0}, a.rho[c]).re;
        if (a.src[1] && i == is && k == ks) vy.re = vy.re + cdiv(cx{(real)a.src[1][it - 1] * dt, 0}, a.rho[c]).re;
        if (a.src[2] && i == is && k == ks + 1) vz.re = vz.re + cdiv(cx{(real)a.src[2][it - 1] * dt, 0}, a.rho[c]).re;
        if (i == 1 || i == nx || k == 1 || k == nz) { vx = cx{0, 0}; vy = cx{0, 0}; vz = cx{0, 0}; }
        stc(a.f[0], c, vx);
        stc(a.f[1], c, vy);
        stc(a.f[2], c, vz);
#if !SD_F32
        const double n1 = (double)vx.re * vx.re + (double)vx.im * vx.im;
        const double n2 = (double)vy.re * vy.re + (double)vy.im * vy.im;
        const double n3 = (double)vz.re * vz.re + (double)vz.im * vz.im;
        nrm = sqrt(n1 + n2 + n3);
#else
        sq = (vx.re * vx.re + vx.im * vx.im) + (vy.re * vy.re + vy.im * vy.im) + (vz.re * vz.re + vz.im * vz.im);
        w[0] = vx.re; w[1] = vx.im; w[2] = vy.re; w[3] = vy.im; w[4] = vz.re; w[5] = vz.im;
#endif
        // plane-wave face cells: their norm is taken after the injection
        if (a.pw.on && pw_cell(a.pw, i - 1, 0, k - 1)) {
            nrm = 0.0; sq = 0.f;
            for (float& x : w) x = 0.f;
        }
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

// stress source, cpmlfdtd.f08:1268-1273 (real parts; applied after the velocity update)
__global__ void s25_stress_source(S25Args<real> a, StepInfo si) {
    const int it = *si.step;
    const int nx = a.nx;
    const int is = a.isrc + 1, ks = a.ksrc + 1;
    auto add = [&](real* f, int fi, int fk, const double* s, int ri, int rk) {
        if (!s) return;
        const size_t c = IX(fi, fk);
        f[2 * c] = f[2 * c] + cdiv(cx{(real)s[it - 1], 0}, a.rho[IX(ri, rk)]).re;
    };
    add(a.f[3], is, ks, a.src[3], is, ks);              // sxx
    add(a.f[4], is + 1, ks, a.src[4], is + 1, ks);      // sxy
    add(a.f[5], is + 1, ks + 1, a.src[5], is + 1, ks);  // sxz: density at (is+1, ks), reference quirk
    add(a.f[6], is, ks, a.src[6], is, ks);              // syy
    add(a.f[7], is, ks + 1, a.src[7], is, ks + 1);      // syz
    add(a.f[8], is, ks, a.src[8], is, ks);              // szz
}

// Receiver gather (after the Dirichlet ring, like the reference's per-step
// snapshot) and advance of the device step counter; always the last
// kernel of a step.
__global__ void s25_epilogue(S25Args<real> a, StepInfo s) {
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

void SD_NAME(launch_seismic25)(const S25Args<real>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h) {
    const dim3 blk(BX, BY), grd((a.nx + BX - 1) / BX, (a.nz + BY - 1) / BY);
    s25_stress<<<grd, blk, 0, st>>>(a);
    if (h) h->fn(h->ctx, 0, "s25_stress");
    s25_velocity<<<grd, blk, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 1, "s25_velocity");
    if (a.stress_src) {
        s25_stress_source<<<1, 1, 0, st>>>(a, s);
        if (h) h->fn(h->ctx, 2, "s25_stress_source");
    }
    if (a.pw.on) pw_seismic25<real>(a, s, st);
    s25_epilogue<<<1, 256, 0, st>>>(a, s);
    if (h) h->fn(h->ctx, 3, "s25_epilogue");
}
