// seismic3_cell.cu -- FP32 3D elastic half-steps, one thread per cell with
// every load issued up front.
//
// Same arithmetic as the FP32 path of seismic3.cu (src/fortran/cpmlfdtd.f08:
// 1761-1992 stress loops, :2014-2127 velocity loops).  What changes is the
// memory schedule, shaped by two measurements on this part:
//   * the kernels are latency bound unless each thread has many loads in
//     flight, so a thread first issues all of its loads -- the 39 velocity
//     stencil points (or 32 stress/density points) with clamped, branch-free
//     indices, and the 33 (10) per-cell arrays -- and only then computes;
//   * HBM rewards concurrently running CTAs that walk contiguous memory, so
//     the grid is ordered x tiles, y tiles, z planes (no z-marching), and the
//     read-once arrays stream with ld.global.cs.
// Stencil neighbours are read through the read-only path (ld.global.nc), so
// a value shared by adjacent cells comes from L1/L2, not HBM, after the first
// read.
#include "s3_velocity.cuh"

namespace {

constexpr int BX = 32, BY = 8;
constexpr int NSLOT = 64;

using namespace s3;

__global__ void __launch_bounds__(BX* BY) s3c_stress(S3Args<float> A) {
    const int gx = blockIdx.x * BX + threadIdx.x, gy = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    if (gx >= nx || gy >= ny) return;
    const bool x14 = gx >= 1 && gx <= nx - 3, x23 = gx >= 2 && gx <= nx - 2;
    const bool y13 = gy >= 2 && gy <= ny - 2, y24 = gy >= 1 && gy <= ny - 3;
    const bool z12 = k >= 2 && k <= nz - 2, z34 = k >= 1 && k <= nz - 3;
    const bool L1 = x14 && y13 && z12, L2 = x23 && y24 && z12, L3 = x23 && y13 && z34, L4 = x14 && y24 && z34;
    if (!(L1 || L2 || L3 || L4)) return;
    const size_t sx = 1, sy = (size_t)nx, sz = (size_t)nx * ny;
    const size_t c = (size_t)gx + sy * gy + sz * k;
    // clamped neighbour offsets (cells that use a neighbour always have it in range)
    const long ox[4] = {(long)cl(gx - 2, 0, nx - 1) - gx, (long)cl(gx - 1, 0, nx - 1) - gx,
                        (long)cl(gx + 1, 0, nx - 1) - gx, (long)cl(gx + 2, 0, nx - 1) - gx};
    const long oy[4] = {((long)cl(gy - 2, 0, ny - 1) - gy) * (long)sy, ((long)cl(gy - 1, 0, ny - 1) - gy) * (long)sy,
                        ((long)cl(gy + 1, 0, ny - 1) - gy) * (long)sy, ((long)cl(gy + 2, 0, ny - 1) - gy) * (long)sy};
    const long oz[4] = {((long)cl(k - 2, 0, nz - 1) - k) * (long)sz, ((long)cl(k - 1, 0, nz - 1) - k) * (long)sz,
                        ((long)cl(k + 1, 0, nz - 1) - k) * (long)sz, ((long)cl(k + 2, 0, nz - 1) - k) * (long)sz};
    (void)sx;
    // ---- loads: 39 stencil points, 21 C_ij, 6 gamma factors, 6 old stresses
    float v[3][13];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        const float* p = A.f[f] + c;
        v[f][0] = __ldg(p);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v[f][1 + q] = __ldg(p + ox[q]);
            v[f][5 + q] = __ldg(p + oy[q]);
            v[f][9 + q] = __ldg(p + oz[q]);
        }
    }
    float C[21], gm[6], so[6];
#pragma unroll
    for (int q = 0; q < 21; ++q) C[q] = __ldcs(A.C[q] + c);
#pragma unroll
    for (int q = 0; q < 6; ++q) gm[q] = __ldcs(A.g[q] + c);
#pragma unroll
    for (int q = 0; q < 6; ++q) so[q] = __ldcs(A.f[3 + q] + c);
    // ---- derivatives: index 0 centre, 1..4 = -2,-1,+1,+2 along the axis
    const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
    float fx[3], bx[3], fy[3], by[3], fz[3], bz[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        const float* a = v[f];
        fx[f] = (27.0f * (a[3] - a[0]) - (a[4] - a[2])) * hx;
        bx[f] = (27.0f * (a[0] - a[2]) - (a[3] - a[1])) * hx;
        fy[f] = (27.0f * (a[7] - a[0]) - (a[8] - a[6])) * hy;
        by[f] = (27.0f * (a[0] - a[6]) - (a[7] - a[5])) * hy;
        fz[f] = (27.0f * (a[11] - a[0]) - (a[12] - a[10])) * hz;
        bz[f] = (27.0f * (a[0] - a[10]) - (a[11] - a[9])) * hz;
    }
    const bool pml = !(A.box.i0 <= gx && gx < A.box.i1 && A.box.j0 <= gy && gy < A.box.j1 && A.box.k0 <= k &&
                       k < A.box.k1);
    const float dt = A.dt;
    const auto CR = [&](int q) { return C[q]; };
    // C index: 0 c11 1 c12 2 c13 3 c14 4 c15 5 c16 6 c22 7 c23 8 c24 9 c25 10 c26
    //          11 c33 12 c34 13 c35 14 c36 15 c44 16 c45 17 c46 18 c55 19 c56 20 c66
    // so / gm order: sigma xx xy xz yy yz zz ; gamma x y z xy yz xz
    if (L1) {
        float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {bz[0], bz[1], bz[2]};
        if (pml) loop_cpml<1>(A, c, ex, ey, ez);
        __stcs(A.f[3] + c, stress_new(CR, so[0], gm[0], 0, 1, 2, 3, 4, 5, dt, ex, ey, ez));
        __stcs(A.f[6] + c, stress_new(CR, so[3], gm[1], 1, 6, 7, 8, 9, 10, dt, ex, ey, ez));
        __stcs(A.f[8] + c, stress_new(CR, so[5], gm[2], 2, 7, 11, 12, 13, 14, dt, ex, ey, ez));
    }
    if (L2) {
        float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {bz[0], bz[1], bz[2]};
        if (pml) loop_cpml<2>(A, c, ex, ey, ez);
        __stcs(A.f[4] + c, stress_new(CR, so[1], gm[3], 5, 10, 14, 17, 19, 20, dt, ex, ey, ez));
    }
    if (L3) {
        float ex[3] = {bx[0], bx[1], bx[2]}, ey[3] = {by[0], by[1], by[2]}, ez[3] = {fz[0], fz[1], fz[2]};
        if (pml) loop_cpml<3>(A, c, ex, ey, ez);
        __stcs(A.f[5] + c, stress_new(CR, so[2], gm[5], 4, 9, 13, 16, 18, 19, dt, ex, ey, ez));
    }
    if (L4) {
        float ex[3] = {fx[0], fx[1], fx[2]}, ey[3] = {fy[0], fy[1], fy[2]}, ez[3] = {fz[0], fz[1], fz[2]};
        if (pml) loop_cpml<4>(A, c, ex, ey, ez);
        __stcs(A.f[7] + c, stress_new(CR, so[4], gm[4], 3, 8, 12, 15, 16, 17, dt, ex, ey, ez));
    }
}

// L2 prefetch for the CTA `dist` tiles later in launch order: stresses,
// velocities, density, and on shell tiles the velocity-loop memories and the
// CPML coefficients (a hint; nothing stays allocated for it)
__device__ __forceinline__ void s3c_velocity_prefetch(const S3Args<float>& A, int dist, int tid) {
    (void)dist;  // A.pfv_d holds it split into tile offsets
    int tx, ty, k;
    if (!tile_ahead(A.pfv_d, tx, ty, k)) return;
    pf_tile_rows(A.f, 9, tx, ty, k, A.nx, A.ny, tid, BX * BY);
    pf_tile_rows(&A.rho, 1, tx, ty, k, A.nx, A.ny, tid, BX * BY);
    if (!tile_in_box(A.box, tx, ty, k, A.nx, A.ny)) {
        pf_tile_rows(A.mem + 36, 9, tx, ty, k, A.nx, A.ny, tid, BX * BY);
        pf_cpml_tile(A, tx, ty, k, tid, BX * BY);
    }
}

template <int MINB>
__global__ void __launch_bounds__(BX* BY, MINB) s3c_velocity(S3Args<float> A, StepInfo si) {
    __shared__ unsigned redu[2 * BX * BY / 32];
    __shared__ double redd[2][BX * BY / 32];
    if (A.prefetch_v > 0) s3c_velocity_prefetch(A, A.prefetch_v, threadIdx.y * BX + threadIdx.x);
    const int it = *si.step;
    const int gx = blockIdx.x * BX + threadIdx.x, gy = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    const int nx = A.nx, ny = A.ny;
    const bool col = gx < nx && gy < ny;
    float vsq = 0.f, ssq = 0.f, w[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (lean_tile(A, blockIdx.x * BX, blockIdx.y * BY, k, true)) velocity_cell<true>(A, it, gx, gy, k, vsq, ssq, w);
    else if (col) velocity_cell<false>(A, it, gx, gy, k, vsq, ssq, w);
    double vn, sn;
    block_norm2_f32<BX * BY / 32>(
        vsq, ssq, [&] { return sqrt((double)w[0] * w[0] + (double)w[1] * w[1] + (double)w[2] * w[2]); },
        [&] {
            const double s1 = w[3], s2 = w[4], s3 = w[5], s4 = w[6], s5 = w[7], s6 = w[8];
            return sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6));
        },
        redu, &redd[0][0], vn, sn);
    if ((threadIdx.x | threadIdx.y) == 0) {
        const int slot = (blockIdx.x + 7 * blockIdx.y + 13 * blockIdx.z) % NSLOT;
        atomic_max_nonneg(A.norms_part + slot, vn);
        atomic_max_nonneg(A.norms_part + NSLOT + slot, sn);
    }
}

// ------------------------------------------------ cell-pair variant
// Each thread updates the two x-adjacent cells (x, x+1), x even, of a
// 32 x 16 tile (16 x 16 threads).  On lean tiles every input comes from an
// aligned float2 load that serves both cells -- 29 loads and their address
// arithmetic per pair instead of 64 -- and the arithmetic per cell is the
// one-cell kernel's; other tiles run the one-cell path for each cell.
// Needs nx even (every pair then starts 8 bytes aligned).
// Warp parts (SUB): warp w (rows 2w, 2w + 1 of the tile) makes the lean test
// for its own 32 x 2 part; the grid's inert box rarely ends on a 16-row
// boundary (its high faces lie one cell short of one, where the half-grid
// C-PML profile reaches), so fewer cells take the one-cell path.  (Parts of
// 16 x 4, 8 pairs x 4 rows per warp, made the x granularity finer too but
// cost more in split rows than they saved: 0.881 against 0.790 ms at 352^3.)
constexpr int PX = 16, PY = 16;     // threads per CTA
constexpr int TPX = 32, TPY = 16;   // cells per tile
constexpr int SPY = 2;              // rows per warp part (SUB)

__device__ __forceinline__ float fmax_bits(float a, float b) {
    // non-negative floats order like their bit patterns; NaN wins
    return __uint_as_float(max(__float_as_uint(a), __float_as_uint(b)));
}

// the lean update of one cell from its stencil values (velocity_cell<true>'s
// expressions); returns the new velocity and the squared norms
__device__ __forceinline__ void vel_lean_cell(float sxx0, float sxxm1, float sxxm2, float sxy0, float sxyym1,
                                              float sxyym2, float sxyp1, float sxyp2, float syy0, float syyp1,
                                              float syyp2, float sxz0, float sxzzm1, float sxzzm2, float sxzp1,
                                              float sxzp2, float syz0, float syzym1, float syzym2, float syzzm1,
                                              float syzzm2, float szz0, float szzp1, float szzp2, float r0, float rxm,
                                              float rxp, float rzm, float rzp, float hx, float hy, float hz,
                                              float dt, int code, float& vx, float& vy, float& vz, float& vsq,
                                              float& ssq) {
    const float byy = inv_mean_f(r0, r0, code);
    {
        const float d1 = (27.0f * (sxx0 - sxxm1) + sxxm2) * hx;
        const float d2 = (27.0f * (sxy0 - sxyym1) + sxyym2) * hy;
        const float d3 = (27.0f * (sxz0 - sxzzm1) + sxzzm2) * hz;
        vx = vx + (d1 * inv_mean_f(r0, rxm, code) + d2 * byy + d3 * inv_mean_f(r0, rzm, code)) * dt;
    }
    {
        const float d1 = (27.0f * (sxyp1 - sxy0) - sxyp2) * hx;
        const float d2 = (27.0f * (syyp1 - syy0) - syyp2) * hy;
        const float d3 = (27.0f * (syz0 - syzzm1) + syzzm2) * hz;
        vy = vy + (d1 * inv_mean_f(r0, rxp, code) + d2 * byy + d3 * inv_mean_f(r0, rzm, code)) * dt;
    }
    {
        const float d1 = (27.0f * (sxzp1 - sxz0) - sxzp2) * hx;
        const float d2 = (27.0f * (syz0 - syzym1) + syzym2) * hy;
        const float d3 = (27.0f * (szzp1 - szz0) - szzp2) * hz;
        vz = vz + (d1 * inv_mean_f(r0, rxp, code) + d2 * byy + d3 * inv_mean_f(r0, rzp, code)) * dt;
    }
    vsq = vx * vx + vy * vy + vz * vz;
    ssq = sxx0 * sxx0 + syy0 * syy0 + szz0 * szz0 + 2.0f * (sxy0 * sxy0 + syz0 * syz0 + sxz0 * sxz0);
}

template <int CODE = 0>
__device__ __forceinline__ void velocity_pair_lean(const S3Args<float>& A, int gx, int gy, int k, float& vsq,
                                                   float& ssq) {
    const long sy = A.nx, sz = (long)A.nx * A.ny;
    const size_t c = (size_t)gx + (size_t)sy * gy + (size_t)sz * k;
    auto L = [&](const float* base, long off) { return __ldg(reinterpret_cast<const float2*>(base + c + off)); };
    const float *Sxx = A.f[3], *Sxy = A.f[4], *Sxz = A.f[5], *Syy = A.f[6], *Syz = A.f[7], *Szz = A.f[8], *R = A.rho;
    const float2 sxx_m = L(Sxx, -2), sxx_0 = L(Sxx, 0);
    const float2 sxy_0 = L(Sxy, 0), sxy_p = L(Sxy, 2), sxy_y1 = L(Sxy, -sy), sxy_y2 = L(Sxy, -2 * sy);
    const float2 sxz_0 = L(Sxz, 0), sxz_p = L(Sxz, 2), sxz_z1 = L(Sxz, -sz), sxz_z2 = L(Sxz, -2 * sz);
    const float2 syy_0 = L(Syy, 0), syy_y1 = L(Syy, sy), syy_y2 = L(Syy, 2 * sy);
    const float2 syz_0 = L(Syz, 0), syz_y1 = L(Syz, -sy), syz_y2 = L(Syz, -2 * sy), syz_z1 = L(Syz, -sz),
                 syz_z2 = L(Syz, -2 * sz);
    const float2 szz_0 = L(Szz, 0), szz_z1 = L(Szz, sz), szz_z2 = L(Szz, 2 * sz);
    const float2 r_m = L(R, -2), r_0 = L(R, 0), r_p = L(R, 2), r_zm = L(R, -sz), r_zp = L(R, sz);
    float2* V0 = reinterpret_cast<float2*>(A.f[0] + c);
    float2* V1 = reinterpret_cast<float2*>(A.f[1] + c);
    float2* V2 = reinterpret_cast<float2*>(A.f[2] + c);
    float2 vx = *V0, vy = *V1, vz = *V2;
    const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
    const float dt = A.dt;
    const int code = CODE ? CODE : A.density_code;
    float vs0, ss0, vs1, ss1;
    // cell x: x-2, x-1 from the pair below, x+1, x+2 from this pair and the next
    vel_lean_cell(sxx_0.x, sxx_m.y, sxx_m.x, sxy_0.x, sxy_y1.x, sxy_y2.x, sxy_0.y, sxy_p.x, syy_0.x, syy_y1.x,
                  syy_y2.x, sxz_0.x, sxz_z1.x, sxz_z2.x, sxz_0.y, sxz_p.x, syz_0.x, syz_y1.x, syz_y2.x, syz_z1.x,
                  syz_z2.x, szz_0.x, szz_z1.x, szz_z2.x, r_0.x, r_m.y, r_0.y, r_zm.x, r_zp.x, hx, hy, hz, dt, code,
                  vx.x, vy.x, vz.x, vs0, ss0);
    // cell x+1
    vel_lean_cell(sxx_0.y, sxx_0.x, sxx_m.y, sxy_0.y, sxy_y1.y, sxy_y2.y, sxy_p.x, sxy_p.y, syy_0.y, syy_y1.y,
                  syy_y2.y, sxz_0.y, sxz_z1.y, sxz_z2.y, sxz_p.x, sxz_p.y, syz_0.y, syz_y1.y, syz_y2.y, syz_z1.y,
                  syz_z2.y, szz_0.y, szz_z1.y, szz_z2.y, r_0.y, r_0.x, r_p.x, r_zm.y, r_zp.y, hx, hy, hz, dt, code,
                  vx.y, vy.y, vz.y, vs1, ss1);
    __stcs(V0, vx);
    __stcs(V1, vy);
    __stcs(V2, vz);
    vsq = fmax_bits(vs0, vs1);
    ssq = fmax_bits(ss0, ss1);
}

// lean test of a TW x TH part of a pair tile (the same rules as lean_tile)
template <int TW, int TH>
__device__ __forceinline__ bool lean_tile_p(const S3Args<float>& A, int x0, int y0, int k) {
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    if (!(x0 >= 2 && x0 + TW - 1 <= nx - 3 && y0 >= 2 && y0 + TH - 1 <= ny - 3 && k >= 2 && k <= nz - 3)) return false;
    if (!(x0 >= A.box.i0 && x0 + TW <= A.box.i1 && y0 >= A.box.j0 && y0 + TH <= A.box.j1 && k >= A.box.k0 &&
          k < A.box.k1))
        return false;
    const int is = A.isrc, js = A.jsrc, ks = A.ksrc;
    if (k >= ks && k <= ks + 1 && is + 1 >= x0 && is < x0 + TW && js + 1 >= y0 && js < y0 + TH) return false;
    if (A.pw.on && pw_tile(A.pw, x0, y0, k, TW, TH)) return false;
    return true;
}

// L2 prefetch for the pair tile `A.pfp_d` tiles later (16 rows per tile)
__device__ __forceinline__ void s3p_velocity_prefetch(const S3Args<float>& A, int tid) {
    int tx, ty, k;
    if (!tile_ahead(A.pfp_d, tx, ty, k)) return;
    if (A.v_reverse) k = A.nz - 1 - k;  // the plane that launch position will update
    for (int half = 0; half < 2; ++half) {
        const int ty8 = 2 * ty + half;  // the two 32 x 8 row blocks of the tile
        pf_tile_rows(A.f, 9, tx, ty8, k, A.nx, A.ny, tid, PX * PY);
        pf_tile_rows(&A.rho, 1, tx, ty8, k, A.nx, A.ny, tid, PX * PY);
        if (!tile_in_box(A.box, tx, ty8, k, A.nx, A.ny)) {
            pf_tile_rows(A.mem + 36, 9, tx, ty8, k, A.nx, A.ny, tid, PX * PY);
            pf_cpml_tile(A, tx, ty8, k, tid, PX * PY);
        }
    }
}

// CODE: the density rule compiled in (1..4; the face buoyancies then fold to
// one expression each), 0 = read at run time
template <int MINB, int CODE = 0, bool SUB = false>
__global__ void __launch_bounds__(PX* PY, MINB) s3p_velocity(S3Args<float> A, StepInfo si) {
    __shared__ unsigned redu[2 * PX * PY / 32];
    __shared__ double redd[2][PX * PY / 32];
    const int tid = threadIdx.y * PX + threadIdx.x;
    if (A.prefetch_v > 0) s3p_velocity_prefetch(A, tid);
    const int it = *si.step;
    // v_reverse: the planes are walked from the top, where the stress
    // kernel that just ran finished, so its last stresses are still in L2
    const int k = A.v_reverse ? A.nz - 1 - (int)blockIdx.z : (int)blockIdx.z;
    const int x0 = blockIdx.x * TPX + 2 * threadIdx.x, gy = blockIdx.y * TPY + threadIdx.y;
    const int nx = A.nx, ny = A.ny;
    float vsq = 0.f, ssq = 0.f;
    static_assert(PX * SPY == 32, "a warp part is one warp's rows");
    const bool lean = SUB ? lean_tile_p<TPX, SPY>(A, blockIdx.x * TPX, blockIdx.y * TPY + SPY * (tid >> 5), k)
                          : lean_tile_p<TPX, TPY>(A, blockIdx.x * TPX, blockIdx.y * TPY, k);
    if (lean) {
        velocity_pair_lean<CODE>(A, x0, gy, k, vsq, ssq);
    } else if (gy < ny) {
        float w[9];
        for (int q = 0; q < 2; ++q) {
            if (x0 + q >= nx) break;
            float vs = 0.f, ss = 0.f;
            velocity_cell<false, LD_NC, CODE>(A, it, x0 + q, gy, k, vs, ss, w);
            vsq = fmax_bits(vsq, vs);
            ssq = fmax_bits(ssq, ss);
        }
    }
    // FP64 fallback (a square at or above 3e38): exact norms of this thread's
    // cells, read back (its own writes) -- a blow-up path
    auto exact = [&](bool stress) {
        double m = 0.0;
        if (gy >= ny) return m;
        for (int q = 0; q < 2; ++q) {
            if (x0 + q >= nx) break;
            if (A.pw.on && pw_cell(A.pw, x0 + q, gy, k)) continue;  // taken after the injection
            const size_t c = (size_t)(x0 + q) + (size_t)nx * ((size_t)gy + (size_t)ny * k);
            double n;
            if (!stress) {
                const double a = A.f[0][c], b = A.f[1][c], d = A.f[2][c];
                n = sqrt(a * a + b * b + d * d);
            } else {
                const double s1 = A.f[3][c], s2 = A.f[6][c], s3 = A.f[8][c], s4 = A.f[4][c], s5 = A.f[7][c],
                             s6 = A.f[5][c];
                n = sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6));
            }
            m = nanmax(m, n);
        }
        return m;
    };
    double vn, sn;
    block_norm2_f32<PX * PY / 32>(vsq, ssq, [&] { return exact(false); }, [&] { return exact(true); }, redu,
                                  &redd[0][0], vn, sn);
    if (tid == 0) {
        const int slot = (blockIdx.x + 7 * blockIdx.y + 13 * blockIdx.z) % NSLOT;
        atomic_max_nonneg(A.norms_part + slot, vn);
        atomic_max_nonneg(A.norms_part + NSLOT + slot, sn);
    }
}

// ------------------------------------------------ fully staged variant
// The velocity half-step with every per-cell input staged in shared memory
// by tensor-tile copies before any thread computes: the five stresses with
// x/y stencils (xx xy xz yy yz) and the density as 40 x 12 halo tiles (from
// x0-4, y0-2), sigma_zz of plane k and the z neighbours (sigma_xz, sigma_yz at
// k-1, k-2; sigma_zz at k+1, k+2; density at k-1, k+1) and the old
// velocities as 32 x 8 tiles: 18 copies, one per lane of warp 0, one
// mbarrier.  Out-of-grid parts of a box read zeros and only feed updates the
// cell does not make.  Only CPML memories and coefficients on shell tiles
// still travel through registers.
constexpr int XV_HW = BX + 8, XV_HH = BY + 4, XV_HB = XV_HW * XV_HH;  // 40 x 12
constexpr int XV_SH = 0;                       // [5][XV_HB]: xx xy xz yy yz
constexpr int XV_RH = 5 * XV_HB;               // [XV_HB]: rho
constexpr int XV_P = 6 * XV_HB;                // plain tiles [12][NTV]
constexpr int NTV = BX * BY;
// plain tile slots
constexpr int P_SZZ = 0, P_XZ1 = 1, P_XZ2 = 2, P_YZ1 = 3, P_YZ2 = 4, P_ZZ1 = 5, P_ZZ2 = 6, P_RM = 7, P_RP = 8, P_V = 9;
constexpr int XV_TOTAL = XV_P + 12 * NTV;
constexpr unsigned XV_BYTES = XV_TOTAL * sizeof(float);  // 23,808
constexpr int WAIT_LAND_V = 1 << 26;  // drain bound on the give-up path (copies read local HBM)

template <bool LEAN>
__device__ __forceinline__ void staged_velocity_cell(const S3Args<float>& A, const float* sm, int it, int gx, int gy,
                                                     int k, int tid, float& vsq, float& ssq, float (&w)[9]) {
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
    const size_t c = (size_t)gx + sy * gy + sz * k;
    const int hc = (threadIdx.y + 2) * XV_HW + threadIdx.x + 4;
    const float *Sxx = sm + XV_SH + hc, *Sxy = sm + XV_SH + XV_HB + hc, *Sxz = sm + XV_SH + 2 * XV_HB + hc,
                *Syy = sm + XV_SH + 3 * XV_HB + hc, *Syz = sm + XV_SH + 4 * XV_HB + hc, *R = sm + XV_RH + hc;
    const float* P = sm + XV_P + tid;
    const float sxx0 = Sxx[0], sxxm1 = Sxx[-1], sxxm2 = Sxx[-2];
    const float sxy0 = Sxy[0], sxyp1 = Sxy[1], sxyp2 = Sxy[2], sxyym1 = Sxy[-XV_HW], sxyym2 = Sxy[-2 * XV_HW];
    const float syy0 = Syy[0], syyp1 = Syy[XV_HW], syyp2 = Syy[2 * XV_HW];
    const float sxz0 = Sxz[0], sxzp1 = Sxz[1], sxzp2 = Sxz[2], sxzzm1 = P[P_XZ1 * NTV], sxzzm2 = P[P_XZ2 * NTV];
    const float syz0 = Syz[0], syzym1 = Syz[-XV_HW], syzym2 = Syz[-2 * XV_HW], syzzm1 = P[P_YZ1 * NTV],
                syzzm2 = P[P_YZ2 * NTV];
    const float szz0 = P[P_SZZ * NTV], szzp1 = P[P_ZZ1 * NTV], szzp2 = P[P_ZZ2 * NTV];
    const float r0 = R[0], rxm = R[-1], rxp = R[1], rzm = P[P_RM * NTV], rzp = P[P_RP * NTV];
    float vx = P[P_V * NTV], vy = P[(P_V + 1) * NTV], vz = P[(P_V + 2) * NTV];
    const float hx = 1.0f / (24.0f * A.dx), hy = 1.0f / (24.0f * A.dy), hz = 1.0f / (24.0f * A.dz);
    const float dt = A.dt;
    const int code = A.density_code;
    const bool pml = !LEAN && !(A.box.i0 <= gx && gx < A.box.i1 && A.box.j0 <= gy && gy < A.box.j1 && A.box.k0 <= k &&
                                k < A.box.k1);
    const float byy = inv_mean_f(r0, r0, code);
    if (LEAN || (gx >= 2 && gx <= nx - 2 && gy >= 2 && gy <= ny - 2 && k >= 2 && k <= nz - 2)) {  // vx
        float d1 = (27.0f * (sxx0 - sxxm1) + sxxm2) * hx;
        float d2 = (27.0f * (sxy0 - sxyym1) + sxyym2) * hy;
        float d3 = (27.0f * (sxz0 - sxzzm1) + sxzzm2) * hz;
        if (pml) {
            const CpmlC p = cpml_at(A, c, true);
            d1 = cpml_apply(A.mem[36], c, p, d1);
            d2 = cpml_apply(A.mem[40], c, p, d2);
            d3 = cpml_apply(A.mem[42], c, p, d3);
        }
        vx = vx + (d1 * inv_mean_f(r0, rxm, code) + d2 * byy + d3 * inv_mean_f(r0, rzm, code)) * dt;
    }
    if (LEAN || (gx >= 1 && gx <= nx - 3 && gy >= 1 && gy <= ny - 3 && k >= 2 && k <= nz - 2)) {  // vy
        float d1 = (27.0f * (sxyp1 - sxy0) - sxyp2) * hx;
        float d2 = (27.0f * (syyp1 - syy0) - syyp2) * hy;
        float d3 = (27.0f * (syz0 - syzzm1) + syzzm2) * hz;
        if (pml) {
            const CpmlC ph = cpml_at(A, c, true), pf = cpml_at(A, c, false);
            d1 = cpml_apply(A.mem[39], c, ph, d1);
            d2 = cpml_apply(A.mem[37], c, ph, d2);
            d3 = cpml_apply(A.mem[44], c, pf, d3);
        }
        vy = vy + (d1 * inv_mean_f(r0, rxp, code) + d2 * byy + d3 * inv_mean_f(r0, rzm, code)) * dt;
    }
    if (LEAN || (gx >= 1 && gx <= nx - 3 && gy >= 2 && gy <= ny - 2 && k >= 1 && k <= nz - 3)) {  // vz
        float d1 = (27.0f * (sxzp1 - sxz0) - sxzp2) * hx;
        float d2 = (27.0f * (syz0 - syzym1) + syzym2) * hy;
        float d3 = (27.0f * (szzp1 - szz0) - szzp2) * hz;
        if (pml) {
            const CpmlC ph = cpml_at(A, c, true), pf = cpml_at(A, c, false);
            d1 = cpml_apply(A.mem[41], c, ph, d1);
            d2 = cpml_apply(A.mem[43], c, pf, d2);
            d3 = cpml_apply(A.mem[38], c, ph, d3);
        }
        vz = vz + (d1 * inv_mean_f(r0, rxp, code) + d2 * byy + d3 * inv_mean_f(r0, rzp, code)) * dt;
    }
    bool src_cell = false;
    if (!LEAN) {
        // force source (cpmlfdtd.f08:2214-2219)
        const int is = A.isrc, js = A.jsrc, ks = A.ksrc;
        if (gx == is + 1 && gy == js && k == ks && A.src[0]) vx = vx + (float)A.src[0][it - 1] * dt / r0;
        if (gx == is && gy == js + 1 && k == ks && A.src[1])
            vy = vy + (float)A.src[1][it - 1] * dt / A.rho[(size_t)is + sy * js + sz * ks];
        if (gx == is && gy == js && k == ks + 1 && A.src[2]) vz = vz + (float)A.src[2][it - 1] * dt / r0;
        if (gx == 0 || gx == nx - 1 || gy == 0 || gy == ny - 1 || k == 0 || k == nz - 1) { vx = 0.f; vy = 0.f; vz = 0.f; }
        src_cell = A.stress_src && ((gx == is && gy == js && k == ks) || (gx == is + 1 && gy == js + 1 && k == ks) ||
                                    (gx == is + 1 && gy == js && k == ks + 1) || (gx == is && gy == js + 1 && k == ks + 1));
    }
    __stcs(A.f[0] + c, vx);
    __stcs(A.f[1] + c, vy);
    __stcs(A.f[2] + c, vz);
    w[0] = vx; w[1] = vy; w[2] = vz;
    vsq = vx * vx + vy * vy + vz * vz;
    if (!src_cell) {
        w[3] = sxx0; w[4] = syy0; w[5] = szz0; w[6] = sxy0; w[7] = syz0; w[8] = sxz0;
        ssq = w[3] * w[3] + w[4] * w[4] + w[5] * w[5] + 2.0f * (w[6] * w[6] + w[7] * w[7] + w[8] * w[8]);
    }
}

__global__ void __launch_bounds__(BX* BY) s3x_velocity(S3Args<float> A, StepInfo si, const __grid_constant__ S3XMaps M) {
    extern __shared__ __align__(128) float sm[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ unsigned redu[2 * BX * BY / 32];
    __shared__ double redd[2][BX * BY / 32];
    const int tid = threadIdx.y * BX + threadIdx.x;
    if (A.prefetch_v > 0) s3c_velocity_prefetch(A, A.prefetch_v, tid);
    const int it = *si.step;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY, k = blockIdx.z;
    const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
    const int nx = A.nx, ny = A.ny;
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_expect_tx(&bar, XV_BYTES);
    }
    __syncthreads();
    if (tid < 18) {  // one copy per lane of warp 0
        if (tid < 5) {
            tma_load3(sm + XV_SH + tid * XV_HB, &M.sigh[tid], x0 - 4, y0 - 2, k, &bar);
        } else if (tid == 5) {
            tma_load3(sm + XV_RH, &M.rhoh, x0 - 4, y0 - 2, k, &bar);
        } else {
            const int q = tid - 6;  // plain slot
            const CUtensorMap* map;
            int z = k;
            switch (q) {
            case P_SZZ: map = &M.sig[5]; break;
            case P_XZ1: map = &M.sig[2]; z = k - 1; break;
            case P_XZ2: map = &M.sig[2]; z = k - 2; break;
            case P_YZ1: map = &M.sig[4]; z = k - 1; break;
            case P_YZ2: map = &M.sig[4]; z = k - 2; break;
            case P_ZZ1: map = &M.sig[5]; z = k + 1; break;
            case P_ZZ2: map = &M.sig[5]; z = k + 2; break;
            case P_RM: map = &M.rhop; z = k - 1; break;
            case P_RP: map = &M.rhop; z = k + 1; break;
            default: map = &M.vp[q - P_V]; break;
            }
            tma_load3(sm + XV_P + q * NTV, map, x0, y0, z, &bar);
        }
    }
    float vsq = 0.f, ssq = 0.f, w[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const bool ok = mbar_wait_bounded(&bar, 0, A.wait_limit);
    if (!ok) {
        if (A.err) atomicExch(A.err, 1);
        if (tid == 0) mbar_wait_bounded(&bar, 0, WAIT_LAND_V);
    } else if (lean_tile(A, x0, y0, k, true)) {
        staged_velocity_cell<true>(A, sm, it, gx, gy, k, tid, vsq, ssq, w);
    } else if (gx < nx && gy < ny) {
        staged_velocity_cell<false>(A, sm, it, gx, gy, k, tid, vsq, ssq, w);
    }
    double vn, sn;
    block_norm2_f32<BX * BY / 32>(
        vsq, ssq, [&] { return sqrt((double)w[0] * w[0] + (double)w[1] * w[1] + (double)w[2] * w[2]); },
        [&] {
            const double s1 = w[3], s2 = w[4], s3 = w[5], s4 = w[6], s5 = w[7], s6 = w[8];
            return sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6));
        },
        redu, &redd[0][0], vn, sn);
    if (tid == 0) {
        const int slot = (blockIdx.x + 7 * blockIdx.y + 13 * blockIdx.z) % NSLOT;
        atomic_max_nonneg(A.norms_part + slot, vn);
        atomic_max_nonneg(A.norms_part + NSLOT + slot, sn);
    }
}

}  // namespace

bool seismic3_staged_velocity_prepare(const S3Args<float>& a, S3XMaps* m) {
    if (a.nx % 4 != 0) return false;
    for (int q = 0; q < 5; ++q)
        if (!seismic3_make_map(&m->sigh[q], a.f[3 + q], a.nx, a.ny, a.nz, XV_HW, XV_HH)) return false;
    if (!seismic3_make_map(&m->rhoh, a.rho, a.nx, a.ny, a.nz, XV_HW, XV_HH)) return false;
    if (!seismic3_make_map(&m->rhop, a.rho, a.nx, a.ny, a.nz, BX, BY)) return false;
    for (int q = 0; q < 6; ++q)
        if (!seismic3_make_map(&m->sig[q], a.f[3 + q], a.nx, a.ny, a.nz, BX, BY)) return false;
    for (int f = 0; f < 3; ++f)
        if (!seismic3_make_map(&m->vp[f], a.f[f], a.nx, a.ny, a.nz, BX, BY)) return false;
    return true;
}

void launch_seismic3_staged_velocity(const S3Args<float>& a, const S3XMaps& maps, const StepInfo& s, cudaStream_t st) {
    s3x_velocity<<<dim3((a.nx + BX - 1) / BX, (a.ny + BY - 1) / BY, a.nz), dim3(BX, BY), XV_BYTES, st>>>(a, s, maps);
}

void launch_seismic3_pair_velocity(const S3Args<float>& a, const StepInfo& s, cudaStream_t st) {
    const dim3 grd((a.nx + TPX - 1) / TPX, (a.ny + TPY - 1) / TPY, a.nz), blk(PX, PY);
    switch (a.velocity_minb) {
    case 5: s3p_velocity<5><<<grd, blk, 0, st>>>(a, s); break;
    case 6: s3p_velocity<6><<<grd, blk, 0, st>>>(a, s); break;
    case 7: s3p_velocity<7><<<grd, blk, 0, st>>>(a, s); break;
    case 8: s3p_velocity<8><<<grd, blk, 0, st>>>(a, s); break;
    default:
        if (a.velocity_sub) {
            switch (a.density_code) {
            case 1: s3p_velocity<4, 1, true><<<grd, blk, 0, st>>>(a, s); break;
            case 2: s3p_velocity<4, 2, true><<<grd, blk, 0, st>>>(a, s); break;
            case 3: s3p_velocity<4, 3, true><<<grd, blk, 0, st>>>(a, s); break;
            case 4: s3p_velocity<4, 4, true><<<grd, blk, 0, st>>>(a, s); break;
            default: s3p_velocity<4, 0, true><<<grd, blk, 0, st>>>(a, s); break;
            }
            break;
        }
        switch (a.density_code) {
        case 1: s3p_velocity<4, 1><<<grd, blk, 0, st>>>(a, s); break;
        case 2: s3p_velocity<4, 2><<<grd, blk, 0, st>>>(a, s); break;
        case 3: s3p_velocity<4, 3><<<grd, blk, 0, st>>>(a, s); break;
        case 4: s3p_velocity<4, 4><<<grd, blk, 0, st>>>(a, s); break;
        default: s3p_velocity<4><<<grd, blk, 0, st>>>(a, s); break;
        }
        break;
    }
}

void launch_seismic3_cell_stress(const S3Args<float>& a, cudaStream_t st) {
    s3c_stress<<<dim3((a.nx + BX - 1) / BX, (a.ny + BY - 1) / BY, a.nz), dim3(BX, BY), 0, st>>>(a);
}
void launch_seismic3_cell_velocity(const S3Args<float>& a, const StepInfo& s, cudaStream_t st) {
    const dim3 grd((a.nx + BX - 1) / BX, (a.ny + BY - 1) / BY, a.nz), blk(BX, BY);
    switch (a.velocity_minb) {
    case 5: s3c_velocity<5><<<grd, blk, 0, st>>>(a, s); break;
    case 6: s3c_velocity<6><<<grd, blk, 0, st>>>(a, s); break;
    case 7: s3c_velocity<7><<<grd, blk, 0, st>>>(a, s); break;
    case 8: s3c_velocity<8><<<grd, blk, 0, st>>>(a, s); break;
    default: s3c_velocity<4><<<grd, blk, 0, st>>>(a, s); break;
    }
}
