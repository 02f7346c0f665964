// kernels.h -- argument blocks and launchers shared by the solver runtime
// (solver.cu) and the per-family kernel files.  Each launcher exists twice,
// suffixed _f64 (drop-in FP64 build) and _f32 (fast FP32 build).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>

struct BoxH {
    int i0, i1, j0, j1, k0, k1;
};

// Optional callback after each kernel launch of a step (used by the
// profiling entry point to record CUDA events between kernels).
struct LaunchHook {
    void (*fn)(void* ctx, int kernel, const char* name);
    void* ctx;
};

// Per-step scalars common to all families.  The 1-based step number lives in
// device memory (*step) and the last kernel of every step increments it, so
// one captured CUDA graph of G steps replays from any starting step.
// Plane-wave injection (planewave.cu): up to three faces of the interior
// box, applied in x, y, z order after the velocity / E update.  0-based
// cells; a face fixes one axis and spans inclusive ranges on the others.
struct PwFace {
    int axis;          // 0: x, 1: y, 2: z
    int fixed;         // index along `axis`
    int lo[3], hi[3];  // inclusive ranges per axis (the fixed axis: fixed..fixed)
};
struct PwDev {
    int on;            // 0: point sources
    int em;            // 1: E/H fields, 0: elastic
    int nface;
    int wavelet;       // 0 gaus0, 1 gaus1, 2 gaus2
    PwFace face[3];
    double p[3], ehat[3], hhat[3], r0[3], loc[3], h[3];
    double v, eta, amp, f0, dt;
};
// true when cell (i, j, k) lies on an injection face: the velocity / E
// kernels leave it out of their max-norms, the injection takes it
__host__ __device__ inline bool pw_cell(const PwDev& pw, int i, int j, int k) {
    for (int f = 0; f < pw.nface; ++f) {
        const PwFace& F = pw.face[f];
        if (i >= F.lo[0] && i <= F.hi[0] && j >= F.lo[1] && j <= F.hi[1] && k >= F.lo[2] && k <= F.hi[2]) return true;
    }
    return false;
}

struct StepInfo {
    int* step;       // device: 1-based number of the step being computed
    int nrec;        // receivers
    const int* rec;  // receiver cell indices (device)
};

// ------------------------------------------------------------- seismic2
// model slots follow S2_* of seidart_gpu.h.  In the FP32 build the gamma
// slots hold 1/(1+gamma dt) and the kappa slots hold 1/kappa.
template <typename T>
struct S2Args {
    int nx, nz, density_code;
    T dx, dz, dt;
    BoxH box;
    const T* m[16];
    T* f[5];
    T* mem[12];
    const double* src[5];  // source series (device, FP64), NULL = zero
    int isrc, jsrc;        // 0-based source cell
    int stress_src;        // 1 if any stress-source series is non-zero
    T* traces;             // [nt][2][nrec]
    double* norms;         // [nt]
    PwDev pw;              // plane-wave source (pw.on = 0: point sources)
};
void launch_seismic2_f64(const S2Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_seismic2_f64x(const S2Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_seismic2_f32(const S2Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);

// ----------------------------------------------------------- electromag2
// Derived coefficient arrays (aEx..eEz, eps11*eps0, eps33*eps0) are built on
// the host in FP64 from the reference's formulas, then cast.
template <typename T>
struct E2Args {
    int nx, nz;
    T dx, dz, dt, dbHy;
    BoxH box;
    const T* c[10];   // aEx bEx dEx eEx aEz bEz dEz eEz e11abs e33abs
    const T* cpml[6]; // kappa kappa_half acoef acoef_half bcoef bcoef_half
    T* f[3];          // Ex Ez Hy
    T* mem[4];
    const double* src[2];
    int isrc, jsrc;
    T* traces;        // [nt][2][nrec]
    double* norms;
    PwDev pw;         // plane-wave source (pw.on = 0: point sources)
};
void launch_electromag2_f64(const E2Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_electromag2_f64x(const E2Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_electromag2_f32(const E2Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);

// Adjoint of one FP32 electromag2 step (adjoint_em.cu).  State arrays, N
// cells each: Ex Ez Hy m_dEx_dz m_dEz_dx m_dHy_dx m_dHy_dz.
struct EmAdjArgs {
    E2Args<float> a;     // FP32 solver arguments (coefficients, CPML, sizes, source cell)
    const float* xp;     // x_{n-1}: [7][N]
    const float* xc;     // x_n
    float* lam;          // adjoint state [7][N]
    float* scr;          // [4][N]: E^T -> Hy gather (z, x), H^T -> E gather (Ex, Ez)
    float* grad;         // [8][N] FP32 sums: aEx bEx dEx eEx aEz bEz dEz eEz
    size_t N;
    const double* srcz;  // Ez source series of the shot (device), NULL = none
    const int* base;     // device: steps before the segment; this step is *base + j
    int j;
    double* gsrc;        // accumulated lambda_Ez(src) * f_n
    const int* rfirst;   // [N] first receiver at a cell (-1: none)
    const int* rnext;    // [nrec] next receiver at the same cell
    const float* dres;   // [nt][2][nrec] receiver residuals, NULL = none
    int nrec;
};
struct EmOopArgs {
    E2Args<float> a;
    const float* in;     // x_{j-1}: [7][N]
    float* out;          // x_j
    size_t N;
    const double* srcz;
    const int* base;
    int j;
};
void em2_adjoint_step(const EmAdjArgs& A, cudaStream_t st);
void em2_adjoint_flush(const EmAdjArgs& A, cudaStream_t st);
void em2_recompute_step(const EmOopArgs& O, cudaStream_t st);

// ------------------------------------------------------------- seismic25
// Complex fields are interleaved (re, im) arrays of T.  The nine face
// densities are pre-averaged on the host exactly as the reference does
// (array_averaging2d, running averages included).
template <typename T>
struct S25Args {
    int nx, nz;
    T dx, dz, dt, ky;
    BoxH box;
    const T* C[21];
    const T* g[6];     // gamma_x y z xy yz xz (FP32: 1/(1+gamma dt))
    const T* cpml[6];  // kappa kappa_half acoef acoef_half bcoef bcoef_half (FP32: 1/kappa)
    const T* rho9[9];  // rhoxx rhoyx rhozx rhoxy rhoyy rhozy rhoxz rhoyz rhozz (FP32: 1/rho)
    const T* rho;      // raw density for the source terms (FP64 path), 1/rho in FP32
    T* f[9];           // complex
    T* mem[30];        // complex
    const double* src[9];
    int isrc, ksrc;
    int stress_src;
    T* traces;         // [nt][3][nrec] complex
    double* norms;
    PwDev pw;         // plane-wave source (pw.on = 0: point sources)
};
void launch_seismic25_f64(const S25Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_seismic25_f64x(const S25Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_seismic25_f32(const S25Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);

// ----------------------------------------------------------- electromag25
template <typename T>
struct E25Args {
    int nx, nz;
    T dx, dz, dt, ky, dtmu;
    BoxH box;
    const T* sig[6];   // s11 s12 s13 s22 s23 s33
    const T* inv[9];   // aEx bEx cEx aEy bEy cEy aEz bEz cEz
    const T* eabs[3];  // eps11, eps22, eps33 times eps0
    const T* cpml[6];
    T* f[6];           // Ex Ey Ez Hx Hy Hz (complex)
    T* mem[8];
    const double* src[3];
    int isrc, ksrc;
    T* traces;         // [nt][3][nrec] complex
    double* norms;
    PwDev pw;         // plane-wave source (pw.on = 0: point sources)
};
void launch_electromag25_f64(const E25Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_electromag25_f64x(const E25Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_electromag25_f32(const E25Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);

// ----------------------------------------------------------- electromag3
// Derived coefficients (aEx .. cEz with the symmetric ones shared, eps_ii *
// eps0 for the sources) are built on the host in FP64 from the reference's
// formulas, then cast.  FP32: dx, dy, dz hold 1/dx, 1/dy, 1/dz and the kappa
// slots 1/kappa.
template <typename T>
struct E3Args {
    int nx, ny, nz;
    T dx, dy, dz, dt, dbH;
    BoxH box;
    const T* sig[6];   // s11 s12 s13 s22 s23 s33
    const T* inv[9];   // aEx bEx cEx aEy bEy cEy aEz bEz cEz
    const T* eabs[3];  // eps11, eps22, eps33 times eps0
    const T* cpml[6];  // kappa kappa_half acoef acoef_half bcoef bcoef_half
    T* f[6];           // Ex Ey Ez Hx Hy Hz
    T* mem[12];        // E3_M_* order
    const double* src[3];
    int isrc, jsrc, ksrc;  // 0-based source cell
    T* traces;         // [nt][3][nrec]
    double* norms;
    PwDev pw;         // plane-wave source (pw.on = 0: point sources)
};
void launch_electromag3_f64(const E3Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_electromag3_f64x(const E3Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_electromag3_f32(const E3Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);

// -------------------------------------------------------------- seismic3
template <typename T>
struct S3Args {
    int nx, ny, nz, density_code;
    T dx, dy, dz, dt;
    BoxH box;
    const T* C[21];
    const T* rho;     // FP64: rho;   FP32: rho (buoyancy computed per face)
    const T* g[6];    // gamma_x y z xy yz xz (FP32: 1/(1+gamma dt))
    const T* cpml[6]; // FP32: kappa slots hold 1/kappa
    T* f[9];
    T* mem[45];
    const double* src[9];
    int isrc, jsrc, ksrc;
    int stress_src;
    T* traces;        // [nt][3][nrec]
    double* norms;    // [2][nt]: velocity norm, stress norm
    PwDev pw;         // plane-wave source (pw.on = 0: point sources)
    int nt;
    double* norms_part;  // [2][64] per-step partial maxima (FP32 z-marching kernels)
    int* err;            // device error word: 1 = a bounded wait gave up
    const float* packed; // FP32: tile-packed 21 C_ij + 6 gamma factors (bulk stress kernel), or NULL
    int bulk_variant;    // FP32: occupancy variant of the bulk stress kernel
    int prefetch;        // FP32: L2 prefetch distance in tiles of the stress kernel (0 = off)
    int prefetch_v;      // FP32: the same for the velocity kernel
    int pf_d[3];         // `prefetch` as tile offsets (x, y, z) on the 32 x 8 x 1 tile grid
    int pfv_d[3];        // the same for `prefetch_v`
    int pfp_d[3];        // the pair velocity kernel's prefetch distance on its 32 x 16 x 1 tile grid
    int velocity_pair;   // FP32: 1 = the cell-pair velocity kernel (nx even)
    int velocity_sub;    // pair velocity kernel: 1 = each warp makes the lean test for its own two rows
    const void* staged;  // host pointer to S3XMaps when the staged stress kernel is set up, else NULL
    const void* staged_v;  // the same for the staged velocity kernel
    int velocity_minb;     // FP32: CTAs per SM the cell velocity kernel is compiled for (4 .. 8)
    int wait_limit;        // FP32: polls of a bounded mbarrier or plane wait before the kernel gives up
    int wait_probe;        // test hook: bytes armed beyond a copy's size on one CTA (0 = off)
    int* wave_ctl;         // FP32 fused step: [0] work ticket, [WAVE_DONE0 + k] tiles of plane k done; NULL = two kernels
    int wave_n;            // ints of wave_ctl the epilogue clears
    int wave_ctas;         // CTAs of the persistent fused step (resident slots)
    int wave_lag;          // planes between the fused step's stress and velocity fronts (0: default)
    int l2_hint;           // FP32 staged stress: 1 = read-once copies with an L2 evict-first policy
    int v_reverse;         // FP32 velocity kernels: 1 = walk the planes from nz-1 down to 0
    // FP32 staged stress kernel, material-indexed model: when the 21 C_ij and
    // 6 attenuation factors take at most S3_MAXMAT distinct tuples, mat_ids
    // holds one byte per cell (tile-packed like `packed`: [tile][8][32]) and
    // mat_tab the tuples ([S3_MAXMAT][27] floats); NULL = per-cell arrays
    const unsigned char* mat_ids;
    const float* mat_tab;
    int mat_tab_bytes;     // bytes of mat_tab a tile copies (a multiple of 16)
    // indexed C-PML coefficients (FP32 staged stress and pair velocity
    // kernels): one byte per cell, tile-packed like mat_ids, and a
    // [S3_MAXCPML][6] table of the six grids' values; NULL = per-cell grids
    const unsigned char* cpml_ids;
    const float* cpml_tab;
    int mem_merged;        // FP32 staged stress kernel: 1 = the 36 stress-loop C-PML memories held as 21
                           // (derivatives two loops share advance one memory; slots 0..17 and 20, 23, 26)
};
constexpr int S3_MAXMAT = 32;
constexpr int S3_MAXCPML = 64;  // C-PML coefficient tuples of the indexed C-PML layout
// The material index of an FP32 3D solver's coefficient arrays, found on the
// device (matidx.cu): on success the tile-packed material bytes and the
// [S3_MAXMAT][27] FP32 table (both cudaMalloc'd, the caller frees them) and
// the number of materials, returned too; 0 when the model holds more than
// S3_MAXMAT distinct tuples (or on an allocation failure).
int seismic3_material_index(const S3Args<float>& a, int nx, int ny, int nz, unsigned char** ids, float** tab,
                            int* nmat, cudaStream_t st);
// The same for the six C-PML coefficient grids (1/kappa, 1/kappa_half, a,
// a_half, b, b_half as stored for FP32): tile-packed bytes and a
// [S3_MAXCPML][6] table, 0 when they hold more than S3_MAXCPML tuples.
int seismic3_cpml_index(const S3Args<float>& a, int nx, int ny, int nz, unsigned char** ids, float** tab, int* ntup,
                        cudaStream_t st);
// The same for the nine stress coefficients of an FP32 seismic2 model
// (c11 c13 c15 c33 c35 c55 and the three attenuation factors, in that order
// in `coef`): one byte per cell in grid order and a [S3_MAXMAT][9] table.
int seismic2_material_index(const float* const* coef, size_t ncell, unsigned char** ids, float** tab, int* nmat,
                            cudaStream_t st);
// layout of S3Args::wave_ctl
constexpr int WAVE_DONE0 = 32;
// TMA tensor maps of the staged FP32 3D stress kernel: old stresses (32 x 8
// boxes), velocities with a 4/2-cell x/y halo (40 x 12 boxes) and without
// (32 x 8 boxes, for the z neighbours)
struct S3XMaps {
    CUtensorMap sig[6];
    CUtensorMap vh[3];
    CUtensorMap vp[3];
    CUtensorMap sigh[5];  // stresses xx xy xz yy yz with the 40 x 12 halo box (velocity kernel)
    CUtensorMap rhoh, rhop;  // density with and without the halo box
};
bool seismic3_staged_velocity_prepare(const S3Args<float>& a, S3XMaps* maps);
void launch_seismic3_staged_velocity(const S3Args<float>& a, const S3XMaps& maps, const StepInfo& s, cudaStream_t st);
bool seismic3_make_map(CUtensorMap* m, const float* base, int nx, int ny, int nz, int bx, int by);
bool seismic3_staged_prepare(const S3Args<float>& a, S3XMaps* maps);
void launch_seismic3_staged_stress(const S3Args<float>& a, const S3XMaps& maps, cudaStream_t st);
// fused step: both half-steps of one time step in one launch (wavefront over z planes)
// resident CTAs of the fused step on this device (0: not available)
int seismic3_wave_prepare(const S3Args<float>& a);
void launch_seismic3_wave(const S3Args<float>& a, const S3XMaps& maps, const StepInfo& s, cudaStream_t st);
// TMA tensor maps of the FP32 3D stress kernel: 33 plane tiles per cell
// (21 C_ij, 6 attenuation factors, 6 old stresses) and the 3 velocity planes
struct S3Maps {
    CUtensorMap coef[33];
    CUtensorMap v[3];
    int variant;  // tile shape / pipeline depth variant the maps were built for
};
// FP32 path of seismic3: kernel families per half-step
enum { S3K_CELL = 0, S3K_ZMARCH = 1, S3K_TMA = 2, S3K_BULK = 3 };
void launch_seismic3_fast(const S3Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h,
                          const S3Maps* maps, int stress_kind, int velocity_kind);
void launch_seismic3_cell_stress(const S3Args<float>& a, cudaStream_t st);
void launch_seismic3_cell_velocity(const S3Args<float>& a, const StepInfo& s, cudaStream_t st);
void launch_seismic3_pair_velocity(const S3Args<float>& a, const StepInfo& s, cudaStream_t st);
int seismic3_fast_norm_slots();
bool seismic3_tma_prepare(const S3Args<float>& a, S3Maps* maps, int variant);
int seismic3_tma_variants();
void seismic3_tma_variant_info(int v, int* tx, int* ty, int* sc, int* rv, int* minb);
void launch_seismic3_tma_stress(const S3Args<float>& a, const S3Maps& maps, cudaStream_t st);
size_t seismic3_bulk_bytes(int nx, int ny, int nz);
int seismic3_bulk_variants();
int seismic3_bulk_variant_minblocks(int v);
cudaError_t seismic3_bulk_pack(const S3Args<float>& a, float* packed, cudaStream_t st);
void launch_seismic3_bulk_stress(const S3Args<float>& a, int variant, cudaStream_t st);
// plane-wave injection and the max-norms of the face cells (planewave.cu),
// launched by each family before its epilogue when a.pw.on
template <typename T> void pw_seismic2(const S2Args<T>& a, const StepInfo& s, cudaStream_t st);
template <typename T> void pw_seismic25(const S25Args<T>& a, const StepInfo& s, cudaStream_t st);
template <typename T> void pw_seismic3(const S3Args<T>& a, const StepInfo& s, cudaStream_t st);
template <typename T> void pw_electromag2(const E2Args<T>& a, const StepInfo& s, cudaStream_t st);
template <typename T> void pw_electromag3(const E3Args<T>& a, const StepInfo& s, cudaStream_t st);
void launch_seismic3_f64(const S3Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_seismic3_f64x(const S3Args<double>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);
void launch_seismic3_f32(const S3Args<float>& a, const StepInfo& s, cudaStream_t st, const LaunchHook* h = nullptr);

// Number of kernel launches one step of each family issues (for accounting).
int seidart_step_launches(int family, int stress_src);
