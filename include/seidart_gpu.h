/*
 * seidart_gpu.h -- C ABI of the GB300 (sm_103a) CPML-FDTD solvers.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns an int status (SEIDART_OK = 0, negative SEIDART_ERR_* on failure;
 * seidart_last_error() gives the message of the calling thread's last error).
 *
 * Grid layout everywhere: Fortran column-major on the PADDED grid, x fastest:
 *   2D / 2.5D : a(i,k)   -> a[i + nx*k]              (0-based i < nx, k < nz)
 *   3D        : a(i,j,k) -> a[i + nx*(j + ny*k)]
 * Padded means n = n_interior + 2*cpml, exactly as the reference pads the grid
 * before calling a solver (src/fortran/main.f08:69-71).  Complex (2.5D) arrays
 * are interleaved (re, im) doubles, the memory layout of Fortran complex(real64).
 *
 * Reference interfaces these calls replace:
 *   seismic2      src/fortran/cpmlfdtd.f08:57-597    (subroutine seismic2)
 *   seismic25     src/fortran/cpmlfdtd.f08:600-1337  (subroutine seismic25)
 *   seismic3      src/fortran/cpmlfdtd.f08:1341-2313 (subroutine seismic3)
 *   electromag2   src/fortran/cpmlfdtd.f08:2317-2760 (subroutine electromag2)
 *   electromag25  src/fortran/cpmlfdtd.f08:2764-3350 (subroutine electromag25)
 *   electromag3   src/fortran/cpmlfdtd.f08:3353-4001 (subroutine electromag3)
 *   legacy names  legacy/cpmlfdtd_wrapper.c:7-16     (seismic2_ ... electromag25c_)
 */
#ifndef SEIDART_GPU_H
#define SEIDART_GPU_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define SEIDART_OK               0
#define SEIDART_ERR_ARG         -1  /* bad argument (sizes, indices, NULL)        */
#define SEIDART_ERR_CUDA        -2  /* CUDA runtime error                         */
#define SEIDART_ERR_UNSTABLE    -3  /* max |v| exceeded 1e25 (reference: stop)    */
#define SEIDART_ERR_IO          -4  /* file contract: missing / malformed record  */
#define SEIDART_ERR_NOMEM       -5  /* device allocation failed                   */
#define SEIDART_ERR_TIMEOUT     -6  /* a bounded device wait gave up              */
#define SEIDART_ERR_UNSUPPORTED -7  /* e.g. plane-wave source, missing GPU        */

/* ------------------------------------------------------- solver families */
#define SEIDART_SEISMIC2      1
#define SEIDART_SEISMIC25     2
#define SEIDART_SEISMIC3      3
#define SEIDART_ELECTROMAG2   4
#define SEIDART_ELECTROMAG25  5
#define SEIDART_ELECTROMAG3   6

/* precision of the field arrays and stencil arithmetic */
#define SEIDART_FP64 0   /* drop-in path: same operation order as the reference */
#define SEIDART_FP32 1   /* fast path: FP32 fields, FP64 set-up of coefficients */
#define SEIDART_FP64_FAST 2  /* FP64 fields with the fast path's arithmetic (host reciprocals,
                                FMA contraction): not bit-identical to the reference's operation
                                order, within 1e-12 relative L2 of it */

/* density face averaging, src/fortran/averaging.f08:5-25 (scalar_mean codes) */
#define SEIDART_DENSITY_HARMONIC   1
#define SEIDART_DENSITY_GEOMETRIC  2
#define SEIDART_DENSITY_ARITHMETIC 3
#define SEIDART_DENSITY_NONE       4

/* Domain_Type (src/fortran/seidart_types.f08:13-20); nx/ny/nz already padded. */
typedef struct SeidartDomain {
    double dim;            /* 2, 2.5 or 3 */
    int nx, ny, nz;        /* padded sizes; ny is ignored in 2D/2.5D */
    double dx, dy, dz;
    int cpml;              /* CPML thickness in cells */
} SeidartDomain;

/* Source_Type (src/fortran/seidart_types.f08:23-33), point sources only. */
typedef struct SeidartSource {
    double dt;
    int time_steps;        /* length of every source time series */
    int xind, yind, zind;  /* interior indices; source cell = ind + cpml (1-based) */
    double ky;             /* 2.5D wavenumber (reference reads env KY) */
} SeidartSource;

/* Plane-wave source parameters (the plane-wave fields of the reference's
 * Source record, src/fortran/seidart_types.f08; plane_wave_source.f08).
 * kind: SEIDART_PW_S for source_type "pw" (elastic also "pws", "pw_s",
 * "pw-s": transverse polarisation), SEIDART_PW_P for "pwp", "pw_p", "pw-p"
 * (elastic only: polarisation along the propagation direction).  wavelet:
 * 0 gaus0 (also any other name), 1 gaus1, 2 gaus2.  Angles in degrees
 * (JSON "x-z_rotation", "x-y_rotation", "y-z_rotation"); frequency is
 * "source_frequency" (Hz), amplitude "amplitude". */
#define SEIDART_PW_S 1
#define SEIDART_PW_P 2
typedef struct SeidartPlaneWave {
    int kind;
    int wavelet;
    double x_z_rotation, x_y_rotation, y_z_rotation;
    double amplitude, frequency;
} SeidartPlaneWave;

/* ---------------------------------------------------------- array slots
 * Host arrays are passed as `const double* const* arrays` in these orders.
 * Model arrays are read-only grids; source series have time_steps entries
 * (NULL = all zeros); field / memory arrays are grids of state.              */

/* C_ij order shared by seismic25 / seismic3 */
enum { SEIDART_C11, SEIDART_C12, SEIDART_C13, SEIDART_C14, SEIDART_C15, SEIDART_C16,
       SEIDART_C22, SEIDART_C23, SEIDART_C24, SEIDART_C25, SEIDART_C26,
       SEIDART_C33, SEIDART_C34, SEIDART_C35, SEIDART_C36,
       SEIDART_C44, SEIDART_C45, SEIDART_C46, SEIDART_C55, SEIDART_C56, SEIDART_C66,
       SEIDART_RHO3,                                   /* 21 */
       SEIDART_GX3, SEIDART_GY3, SEIDART_GZ3,          /* gamma_x, gamma_y, gamma_z    */
       SEIDART_GXY3, SEIDART_GYZ3, SEIDART_GXZ3,       /* gamma_xy, gamma_yz, gamma_xz */
       SEIDART_KAPPA3, SEIDART_KAPPAH3, SEIDART_ACOEF3, SEIDART_ACOEFH3,
       SEIDART_BCOEF3, SEIDART_BCOEFH3,
       SEIDART_NMODEL3 };                              /* 34 */

/* seismic2 model (src/fortran/cpmlfdtd.f08:159-174, :253-261) */
enum { S2_C11, S2_C13, S2_C15, S2_C33, S2_C35, S2_C55, S2_RHO,
       S2_GX, S2_GZ, S2_GXZ,
       S2_KAPPA, S2_KAPPAH, S2_ACOEF, S2_ACOEFH, S2_BCOEF, S2_BCOEFH,
       S2_NMODEL };                                    /* 16 */
enum { S2_SRCX, S2_SRCZ, S2_SRCXX, S2_SRCXZ, S2_SRCZZ, S2_NSRC };
enum { S2_VX, S2_VZ, S2_SXX, S2_SZZ, S2_SXZ, S2_NFIELD };
enum { S2_M_DVX_DX1, S2_M_DVX_DZ1, S2_M_DVZ_DX1, S2_M_DVZ_DZ1,
       S2_M_DVX_DX2, S2_M_DVX_DZ2, S2_M_DVZ_DX2, S2_M_DVZ_DZ2,
       S2_M_DSXX_DX, S2_M_DSZZ_DZ, S2_M_DSXZ_DX, S2_M_DSXZ_DZ, S2_NMEM };

/* seismic25 / seismic3 sources and fields */
enum { S3_SRCX, S3_SRCY, S3_SRCZ, S3_SRCXX, S3_SRCXY, S3_SRCXZ,
       S3_SRCYY, S3_SRCYZ, S3_SRCZZ, S3_NSRC };
enum { S3_VX, S3_VY, S3_VZ, S3_SXX, S3_SXY, S3_SXZ, S3_SYY, S3_SYZ, S3_SZZ, S3_NFIELD };
/* seismic25 memories: 4 stress loops x {dvx,dvy,dvz} x {dx,dz}, then 6 velocity
 * memories (src/fortran/cpmlfdtd.f08:650-664).  Loop L (1..4) occupies slots
 * 6*(L-1) + {dvx_dx, dvy_dx, dvz_dx, dvx_dz, dvy_dz, dvz_dz}.               */
enum { S25_M_DSXX_DX = 24, S25_M_DSXZ_DZ, S25_M_DSXY_DX, S25_M_DSYZ_DZ,
       S25_M_DSXZ_DX, S25_M_DSZZ_DZ, S25_NMEM };       /* 30 complex */
/* seismic3 memories: 4 stress loops x 9 (dvx_dx,dvx_dy,dvx_dz, dvy_dx,..,dvz_dz)
 * at slot 9*(L-1) + 3*comp + dir, then 9 velocity memories.                 */
enum { S3_M_DSXX_DX = 36, S3_M_DSYY_DY, S3_M_DSZZ_DZ, S3_M_DSXY_DX, S3_M_DSXY_DY,
       S3_M_DSXZ_DX, S3_M_DSXZ_DZ, S3_M_DSYZ_DY, S3_M_DSYZ_DZ, S3_NMEM };  /* 45 */

/* electromag2 (src/fortran/cpmlfdtd.f08:2409-2414, :2484-2491) */
enum { E2_E11, E2_E13, E2_E33, E2_S11, E2_S13, E2_S33,
       E2_KAPPA, E2_KAPPAH, E2_ACOEF, E2_ACOEFH, E2_BCOEF, E2_BCOEFH, E2_NMODEL };
enum { E2_SRCX, E2_SRCZ, E2_NSRC };
enum { E2_EX, E2_EZ, E2_HY, E2_NFIELD };
enum { E2_M_DEX_DZ, E2_M_DEZ_DX, E2_M_DHY_DX, E2_M_DHY_DZ, E2_NMEM };

/* electromag25 (src/fortran/cpmlfdtd.f08:2886-2900) */
enum { E25_E11, E25_E12, E25_E13, E25_E22, E25_E23, E25_E33,
       E25_S11, E25_S12, E25_S13, E25_S22, E25_S23, E25_S33,
       E25_KAPPA, E25_KAPPAH, E25_ACOEF, E25_ACOEFH, E25_BCOEF, E25_BCOEFH,
       E25_NMODEL };
enum { E25_SRCX, E25_SRCY, E25_SRCZ, E25_NSRC };
enum { E25_EX, E25_EY, E25_EZ, E25_HX, E25_HY, E25_HZ, E25_NFIELD };
enum { E25_M_DEY_DX, E25_M_DEY_DZ, E25_M_DEX_DZ, E25_M_DEZ_DX,
       E25_M_DHZ_DX, E25_M_DHX_DZ, E25_M_DHY_DZ, E25_M_DHY_DX, E25_NMEM };

/* electromag3 (src/fortran/cpmlfdtd.f08:3353-4001): relative permittivity
 * e11..e33 and conductivity s11..s33 tensors, CPML coefficients; sources x y
 * z; fields Ex Ey Ez Hx Hy Hz; the 12 memories in the reference's declaration
 * order (:3392-3397) */
enum { E3_E11, E3_E12, E3_E13, E3_E22, E3_E23, E3_E33,
       E3_S11, E3_S12, E3_S13, E3_S22, E3_S23, E3_S33,
       E3_KAPPA, E3_KAPPAH, E3_ACOEF, E3_ACOEFH, E3_BCOEF, E3_BCOEFH,
       E3_NMODEL };
enum { E3_SRCX, E3_SRCY, E3_SRCZ, E3_NSRC };
enum { E3_EX, E3_EY, E3_EZ, E3_HX, E3_HY, E3_HZ, E3_NFIELD };
enum { E3_M_DEX_DY, E3_M_DEY_DX, E3_M_DEX_DZ, E3_M_DEZ_DX, E3_M_DEZ_DY, E3_M_DEY_DZ,
       E3_M_DHZ_DX, E3_M_DHX_DZ, E3_M_DHZ_DY, E3_M_DHY_DZ, E3_M_DHX_DY, E3_M_DHY_DX, E3_NMEM };

/* Number of slots of each kind for a solver family; *is_complex = 1 for 2.5D.
 * *nrec_comp = number of receiver components recorded per receiver and step. */
int seidart_layout(int family, int* nmodel, int* nsrc, int* nfield, int* nmem,
                   int* is_complex, int* nrec_comp);

/* ------------------------------------------------------- one-call runs
 * Run `src->time_steps` steps of a solver from the given initial fields, all
 * buffers on the HOST (copies are done inside).  Mirrors one call of the
 * reference subroutine, minus its file I/O:
 *   fields  in: initial fields (velocity / E initial conditions, the rest
 *               usually zero);  out: fields after the last step.
 *   rec_cells   nrec 0-based linear cell indices (may be 0 / NULL).
 *   traces      out, [time_steps][nrec_comp][nrec] doubles (complex: 2x).
 *   norms       out, [time_steps] max-norm series (3D: [2][time_steps],
 *               velocity then stress norm), may be NULL.
 * Returns SEIDART_ERR_UNSTABLE when the norm exceeds 1e25 (the step is
 * reported by seidart_last_error()), as the reference's `stop` does.        */
int seidart_run(int family, int precision, const SeidartDomain* dom,
                const SeidartSource* src, int density_code,
                const double* const* model, const double* const* srcfn,
                double* const* fields, int nrec, const int* rec_cells,
                double* traces, double* norms);

/* ------------------------------------------------------- solver handles
 * A handle owns the device copy of one model and its state on one CUDA
 * stream; steps are asynchronous on that stream.                           */
typedef struct SeidartSolver SeidartSolver;

/* model[q] are host FP64 grids, except that for seismic2 and seismic3 the
 * stiffness, density and attenuation slots (every slot before the CPML
 * ones) may be DEVICE FP64 grids, e.g. from seidart_stiffness_arrays_dev:
 * those are copied (FP64) or converted (FP32) device to device into the
 * solver's arena.  Any other slot in device memory returns SEIDART_ERR_ARG. */
int seidart_solver_create(SeidartSolver** out, int family, int precision,
                          const SeidartDomain* dom, const SeidartSource* src,
                          int density_code, const double* const* model,
                          const double* const* srcfn, int nrec,
                          const int* rec_cells);
/* Use a caller-owned cudaStream_t (passed as void*; NULL = the handle's own). */
int seidart_solver_set_stream(SeidartSolver* s, void* stream);
int seidart_solver_set_fields(SeidartSolver* s, const double* const* fields);
/* Switch the solver to a plane-wave source (pw != NULL; pw->kind 0 switches
 * back to point sources): the injection faces, polarisation and background
 * speed are set up from the parameters and the host model (the family's
 * slots, as given to seidart_solver_create: the speed comes from the
 * stiffness / permittivity eigenvalues over the grid).  The point-source
 * series are not applied while the plane wave is on (the reference loads
 * none); electromag25 sets the plane wave up but, like the reference
 * (cpmlfdtd.f08:3261-3266), never injects it.
 * Replaces: the plane-wave branches of cpmlfdtd.f08 (seismic2 :186-227,
 * :452-512; seismic25 :802-834, :1207-1260; seismic3 :1548-1606,
 * :2133-2203; electromag2 :2436-2476, :2626-2673; electromag3 :3523-3578,
 * :3833-3900) and plane_wave_source.f08. */
int seidart_solver_set_plane_wave(SeidartSolver* s, const SeidartPlaneWave* pw, const double* const* model);
/* The set-up figures of a plane wave without a solver (host only): out[0]
 * background speed, out[1] impedance (EM; 0 elastic), out[2..4] direction
 * p, out[5..7] polarisation ehat, out[8] number of injection faces,
 * out[9..11] their axes (0 x, 1 y, 2 z; -1 unused), out[12..14] their
 * 0-based fixed indices.  No reference counterpart (the reference keeps these
 * in locals of each solver). */
int seidart_plane_wave_setup(int family, const SeidartDomain* dom, const SeidartSource* src,
                             const SeidartPlaneWave* pw, const double* const* model, double* out);
int seidart_solver_get_fields(SeidartSolver* s, double* const* fields);
/* CPML memory variables expanded to full grids (zeros where not stored). */
int seidart_solver_get_memory(SeidartSolver* s, double* const* mem);
/* Advance nsteps steps (asynchronous). */
int seidart_solver_step(SeidartSolver* s, int nsteps);
/* Wait for the stream; returns SEIDART_ERR_UNSTABLE if any step blew up. */
int seidart_solver_sync(SeidartSolver* s);
/* Copy traces / norms of steps [0, steps_done) to the host. */
int seidart_solver_traces(SeidartSolver* s, double* traces, double* norms);
int seidart_solver_steps_done(const SeidartSolver* s);
/* Materials of an FP32 seismic3 solver's material-indexed coefficient
 * layout: when the 21 stiffness and 6 attenuation arrays hold at most 32
 * distinct tuples (as a model expanded from a material image does), the
 * stress kernel reads one byte per cell and a table instead of 27 arrays,
 * with the same FP32 values (the index is found on the device at set-up).
 * 0 = per-cell arrays (too many tuples, nx not a multiple of 4, another
 * family or precision, or SEIDART_S3_MATIDX=0). */
int seidart_solver_material_count(const SeidartSolver* s);
/* Stress-loop C-PML memory arrays a seismic3 solver advances: 21 when the
 * FP32 staged stress kernel shares one memory between the two loops that
 * apply the same derivative stencil with the same coefficients (the default;
 * SEIDART_S3_MERGE=0 keeps 36), else 36; 0 for other families.
 * seidart_solver_get_memory returns the reference's 36 either way. */
int seidart_solver_stress_memory_arrays(const SeidartSolver* s);
/* Tuples of an FP32 seismic3 solver's indexed C-PML coefficients: when the
 * six C-PML grids hold at most 64 distinct tuples (grids built from 1D
 * damping profiles do), the stress and velocity kernels read one byte per
 * cell and a table instead of six grids, with the same FP32 values.  0 =
 * the grids (too many tuples, nx not a multiple of 4, or
 * SEIDART_S3_CPMLIDX=0). */
int seidart_solver_cpml_tuples(const SeidartSolver* s);
/* Device pointer of field slot `slot` (FP64 or FP32 per precision). */
void* seidart_solver_field_ptr(SeidartSolver* s, int slot);
/* Advance nsteps steps launching kernels one by one (no CUDA graph) with a
 * CUDA event after each kernel, then wait.  Outputs, per kernel slot k of a
 * step (at most 8): kernel_ms[k] summed milliseconds, kernel_launches[k]
 * launches, names + k*names_len its kernel name; *total_ms = elapsed time of
 * the whole run.  Any output pointer may be NULL. */
int seidart_solver_profile(SeidartSolver* s, int nsteps, double* total_ms, double* kernel_ms,
                           int* kernel_launches, char* names, int names_len);
/* Number of kernel launches the last seidart_solver_step call issued. */
long long seidart_solver_launches(const SeidartSolver* s);
/* Diagnostic, no counterpart in the reference (its only failure channel is
 * the blow-up stop, cpmlfdtd.f08:2263): the FP32 3D kernels' bound on each
 * device wait (shared-memory copies, and the fused step's wait for finished
 * planes), in polls; default 2^20.  probe_bytes > 0 (a multiple of 16) is a
 * test hook: one CTA arms its copy barrier with that many bytes more than its
 * copies bring, and one item of the fused step waits for a plane count that
 * is never reached, so those waits run out; the next seidart_solver_sync
 * returns SEIDART_ERR_TIMEOUT once and the solver stays usable. */
int seidart_solver_set_wait(SeidartSolver* s, int limit, int probe_bytes);
int seidart_solver_destroy(SeidartSolver* s);
/* Device pointer, element type and stream of field slot `slot` (for callers
 * that read the live fields on the device, e.g. snapshot writers). */
int seidart_solver_snapshot_source(SeidartSolver* s, int slot, void** dev, int* is_complex,
                                   int* is_fp32, size_t* ncell, void** stream);

const char* seidart_last_error(void);

/* ------------------------------------------------------- file contract
 * The body of the reference subroutines with their file I/O: read every
 * input record from directory `dir` (c11.dat ..., *_cpml.dat,
 * initialcondition*.dat, seismicsource*.dat / electromagneticsource*.dat;
 * src/fortran/seidartio.f08:161-292), run all time steps and write the
 * per-step snapshots Vx|Vy|Vz|Ex|Ey|Ez.<it:06d>.<xind>[.<yind>].<zind>.dat
 * (float32 records if single_output, else float64; seidartio.f08:366-426)
 * and, for 3D, velocity_norm.dat / stress_norm.dat.  The 2.5D solvers write
 * zstd blocks instead unless FDTD_LEGACY_OUTPUT=TRUE: S25.|EM25.<first:06d>-
 * <last:06d>.<xind>.<yind>.<zind>.blk.zst, float32 (x, 1, z, component, step)
 * of the real parts with the CPML stripped, FDTD_STEPS_PER_BLOCK steps per
 * file (default about 2 GiB, at most 500; seidartio.f08:462-734).
 * source_type "ac" loads the force components, any other the stress
 * components (seismic); "pw" (plane wave) returns SEIDART_ERR_UNSUPPORTED.
 * Replaces: seismic2/25/3, electromag2/25/3 in src/fortran/cpmlfdtd.f08. */
int seidart_run_files(const char* dir, int family, int precision, const SeidartDomain* dom,
                      const SeidartSource* src, int density_code, const char* source_type,
                      int single_output, int write_snapshots);
/* The same with the plane-wave parameters of the run (used when
 * source_type names a plane wave: "pw" for every family, and for the
 * elastic ones "pws", "pw_s", "pw-s", "pwp", "pw_p", "pw-p"; the source
 * series files are then not read).  pw may be NULL for point sources. */
int seidart_run_files_pw(const char* dir, int family, int precision, const SeidartDomain* dom,
                         const SeidartSource* src, int density_code, const char* source_type,
                         int single_output, int write_snapshots, const SeidartPlaneWave* pw);
const char* seidart_io_last_error(void);
/* Write one zstd frame holding `bytes` of data: compressed at level 3 by the
 * system libzstd when it can be loaded (as write_zstd_block does,
 * seidartio.f08:528-585), else as raw (stored) zstd blocks; SEIDART_ZSTD_RAW=1
 * forces raw blocks.  The 2.5D block writer uses it. */
int seidart_zstd_write(const char* path, const void* data, size_t bytes);

/* Legacy entry points with the argument layout of legacy/cpmlfdtd_wrapper.c:7-16
 * (padded nx[,ny],nz; spacings; PML thickness; src = interior source indices;
 * number of steps; single-precision output flag).  They read the .dat inputs
 * from the working directory and write the snapshots there; dt follows the
 * legacy rule (legacy/cpmlfdtd_cbindings.f95:867-868 for the elastic case). */
void seismic2_(int nx, int nz, double dx, double dz, int npoints_pml, int* src, int nstep, int single_output);
void seismic25_(int nx, int ny, int nz, double dx, double dy, double dz, int npoints_pml, int* src,
                int nstep, int single_output);
void electromag2_(int nx, int nz, double dx, double dz, int npoints_pml, int* src, int nstep, int single_output);
void electromag25_(int nx, int ny, int nz, double dx, double dy, double dz, int npoints_pml, int* src,
                   int nstep, int single_output);
void electromag2c_(int nx, int nz, double dx, double dz, int npoints_pml, int* src, int nstep, int single_output);
void electromag25c_(int nx, int ny, int nz, double dx, double dy, double dz, int npoints_pml, int* src,
                    int nstep, int single_output);

/* `seidartfdtd <input.json> [seismic=true|false] [density_method=...]`
 * (src/fortran/main.f08:31-119); returns the process exit status. */
int seidart_cli_main(int argc, char** argv);

/* ---- batched 2D elastic runs (FP32).  No counterpart in the reference,
 * which runs one model per process call (seismic2, cpmlfdtd.f08:311-576).
 * nmodels independent seismic2 problems of any grid sizes advance together
 * in one persistent cooperative launch per chunk of steps (captured in a
 * CUDA graph); each model's arrays follow seidart_solver_create.  Grid-wide
 * waits are bounded: seidart_batch_sync returns SEIDART_ERR_TIMEOUT when a
 * barrier gave up.  autotune times every (tile shape, CTAs per SM) variant
 * for trial_steps steps and keeps the fastest. */
typedef struct SeidartBatch SeidartBatch;
int seidart_batch_create(SeidartBatch** out, int nmodels, const SeidartDomain* doms, const SeidartSource* srcs,
                         const int* density_codes, const double* const* const* models,
                         const double* const* const* srcfn, const int* nrec, const int* const* rec_cells);
int seidart_batch_autotune(SeidartBatch* b, int trial_steps, int* best_variant, int* best_bps);
int seidart_batch_tuning(const SeidartBatch* b, int variant, int* tx, int* ty, int* bps, double* ms);
int seidart_batch_set_config(SeidartBatch* b, int variant, int bps);
int seidart_batch_step(SeidartBatch* b, int nsteps, int chunk);
int seidart_batch_sync(SeidartBatch* b);
int seidart_batch_force_timeout(SeidartBatch* b, long long spin_limit);
SeidartSolver* seidart_batch_model(SeidartBatch* b, int m);
int seidart_batch_steps_done(const SeidartBatch* b);
long long seidart_batch_launches(const SeidartBatch* b);
/* How many of the last seidart_batch_step call's launches were replays of a
 * captured CUDA graph (each chunk's persistent launch is captured once per
 * chunk length and configuration; the device may refuse capture of a
 * cooperative launch, in which case the chunks launch directly). */
long long seidart_batch_graph_launches(const SeidartBatch* b);
int seidart_batch_config(const SeidartBatch* b, int* tx, int* ty, int* bps, int* grid);
int seidart_batch_num_variants(void);
/* Materials of model m's indexed stress coefficients: a model whose nine
 * stress coefficients (c11 c13 c15 c33 c35 c55, three attenuation factors)
 * hold at most 32 distinct tuples is walked with one byte per cell and a
 * table of the tuples (found on the device at creation, the same FP32
 * values); 0 = per-cell arrays (or SEIDART_BATCH_MATIDX=0), -1 = bad m. */
int seidart_batch_material_count(const SeidartBatch* b, int m);
/* How kernel variant `variant` walks the flattened tile list: "strided"
 * (CTA b of G takes tiles b, b+G, ...) or "chunked" (a contiguous range per
 * CTA); NULL outside 0 .. seidart_batch_num_variants()-1. */
const char* seidart_batch_variant_walk(int variant);
int seidart_batch_destroy(SeidartBatch* b);
const char* seidart_batch_last_error(void);

/* ---- misfit gradient of the 2D elastic solver (full-waveform inversion).
 * No counterpart in the reference, which runs forward models only.  For
 * L = 1/2 sum_shots sum_steps sum_receivers |v - d|^2 (vx and vz traces of
 * the FP32 solver against observed data), seidart_fwi_gradient returns L and
 * dL/d{c11, c13, c33, c55, rho} on the padded grid ([5][nx*nz] FP64, x
 * fastest) from a hand-written discrete adjoint of the FP32 time loop with
 * FP64 gradient accumulation and sqrt(nt) checkpointing (checkpoint_every =
 * 0 picks ceil(sqrt(time_steps))).  model: S2_* slots as for
 * seidart_solver_create; shots: interior force positions (xind, zind as in
 * SeidartSource) and vertical-force series; observed[s]: [time_steps][2][nrec]
 * (NULL = zeros).  grad may be NULL (loss only). */
typedef struct SeidartFwi SeidartFwi;
int seidart_fwi_create(SeidartFwi** out, const SeidartDomain* dom, const SeidartSource* src, int density_code,
                       const double* const* model, int nshots, const int* shot_xind, const int* shot_zind,
                       const double* const* shot_srcz, int nrec, const int* rec_cells,
                       const double* const* observed, int checkpoint_every);
/* Same for family = SEIDART_SEISMIC2 (as above) or SEIDART_ELECTROMAG2: model
 * E2_* slots (density_code ignored), shot series drive Ez at the shot's cell,
 * traces are Ex and Ez, and seidart_fwi_gradient returns [6][nx*nz]
 * dL/d{eps11, eps13, eps33, sig11, sig13, sig33} (relative permittivities as
 * in e11.dat, conductivities as in s11.dat) through the same checkpointed
 * adjoint of the FP32 electromag2 step (cpmlfdtd.f08:2519-2748). */
int seidart_fwi_create_family(SeidartFwi** out, int family, const SeidartDomain* dom, const SeidartSource* src,
                              int density_code, const double* const* model, int nshots, const int* shot_xind,
                              const int* shot_zind, const double* const* shot_srcz, int nrec, const int* rec_cells,
                              const double* const* observed, int checkpoint_every);
int seidart_fwi_gradient(SeidartFwi* f, double* loss, double* grad);
/* synthetic traces of every shot for the model: [nshots][time_steps][2][nrec] */
int seidart_fwi_model_traces(SeidartFwi* f, double* traces);
/* test hooks on one step with the source off; states are [ns][nx*nz] FP32:
 * seismic2 ns = 17 (vx vz sigmaxx sigmazz sigmaxz, then the 12 memory arrays
 * in S2_M_* order), electromag2 ns = 7 (Ex Ez Hy, then E2_M_* order) */
int seidart_fwi_forward_step_host(SeidartFwi* f, float* x);
int seidart_fwi_adjoint_step_host(SeidartFwi* f, const float* xprev, const float* xcur, float* lam);
long long seidart_fwi_launches(const SeidartFwi* f);
/* seismic2 only: on != 0 makes seidart_fwi_gradient also return dL/dc15 and
 * dL/dc35 after the five above ([7][nx*nz]: c11 c13 c33 c55 rho c15 c35).
 * Both coefficients enter the normal and shear stress updates
 * (cpmlfdtd.f08:342-351, :380-383); their sums cost two more FP32
 * accumulators per cell and adjoint step, so they are off by default. */
int seidart_fwi_set_full_tensor(SeidartFwi* f, int on);
int seidart_fwi_checkpointing(const SeidartFwi* f, int* every, int* count);
int seidart_fwi_destroy(SeidartFwi* f);
const char* seidart_fwi_last_error(void);

/* ---- material pre-pass: material-ID image -> padded coefficient grids.
 * Replaces stiffness_write / attenuation_write / permittivity_write[_c]
 * (legacy/cpmlfdtd_cbindings.f95:60-611), whose C prototypes
 * (legacy/cpmlfdtd_wrapper.c:7-10) pass the Fortran assumed-shape table as a
 * bare pointer and drop stiffness_write's gradient argument, so the table's
 * row count is an explicit argument here.
 *   im:    [nz][nx] int32, x fastest: 1-based row numbers of the table
 *   table: row-major [nmat][ncol] (complex: [nmat][ncol][re, im])
 *          stiffness columns 2..23 = c11 c12 c13 c14 c15 c16 c22 c23 c24 c25
 *          c26 c33 c34 c35 c36 c44 c45 c46 c55 c56 c66 rho; permittivity
 *          columns 2..7 = eps11 12 13 22 23 33, 8..13 = sig11 12 13 22 23 33;
 *          attenuation columns 1..3 = gamma_x gamma_y gamma_z
 * Outputs are padded (nx+2 npml) x (nz+2 npml) FP64 grids, x fastest, with
 * the interior values carried into the CPML in the reference's statement
 * order (its corner and sig12/sig23 edge values included); attenuation leaves
 * cpmlvalue in the CPML.  *_arrays fill caller buffers (out[q] may be NULL to
 * skip one: 22 stiffness grids c11..c66, rho; 12 permittivity grids eps11
 * eps12 eps13 eps22 eps23 eps33 sig11 .. sig33, the eps ones complex
 * interleaved in the _c variant; 3 attenuation grids); *_write write the
 * reference's .dat records (c11.dat … rho.dat, eps11.dat … sig33.dat,
 * gamma_x.dat …) into `dir`.  gradient: [nz][nx] factor applied to the
 * interior density, or NULL for none. */
int seidart_stiffness_arrays(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                             const double* gradient, double* const* out);
int seidart_stiffness_write(const char* dir, const int* im, int nx, int nz, const double* mlist, int nmat, int ncol,
                            int npml, const double* gradient);
int seidart_permittivity_arrays(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                                double* const* out);
int seidart_permittivity_write(const char* dir, const int* im, int nx, int nz, const double* mlist, int nmat,
                               int ncol, int npml);
int seidart_permittivity_arrays_c(const int* im, int nx, int nz, const double* mlist_c, int nmat, int ncol, int npml,
                                  double* const* out);
int seidart_permittivity_write_c(const char* dir, const int* im, int nx, int nz, const double* mlist_c, int nmat,
                                 int ncol, int npml);
int seidart_attenuation_arrays(const int* im, int nx, int nz, const double* alist, int nmat, int ncol, int npml,
                               double cpmlvalue, double* const* out);
int seidart_attenuation_write(const char* dir, const int* im, int nx, int nz, const double* alist, int nmat, int ncol,
                              int npml, double cpmlvalue);
/* The same pre-pass on the device (legacy/cpmlfdtd_cbindings.f95:60-611, as
 * above): dev_out[q] are DEVICE buffers of the padded FP64 grids (every one
 * of the 22 / 12 / 3 is required, since the carry reads them; complex eps
 * grids hold interleaved pairs); im, the table and gradient are host arrays
 * (uploaded to scratch the call allocates and frees).  A fill kernel and one
 * row and one column kernel per carry iteration run on `stream` (a
 * cudaStream_t, NULL = legacy default); the call returns after the stream
 * has finished them.  The grids equal the host pass's bit for bit; a
 * seismic2 / seismic3 solver can take them directly as model arrays (see
 * seidart_solver_create). */
int seidart_stiffness_arrays_dev(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                                 const double* gradient, double* const* dev_out, void* stream);
int seidart_permittivity_arrays_dev(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                                    double* const* dev_out, void* stream);
int seidart_permittivity_arrays_c_dev(const int* im, int nx, int nz, const double* mlist_c, int nmat, int ncol,
                                      int npml, double* const* dev_out, void* stream);
int seidart_attenuation_arrays_dev(const int* im, int nx, int nz, const double* alist, int nmat, int ncol, int npml,
                                   double cpmlvalue, double* const* dev_out, void* stream);

/* ---- trace misfit without device allocation.  No counterpart in the
 * reference (SeidarT-Backend computes no misfit); it is the no-allocation
 * variant of the misfit reduction inside seidart_fwi_gradient, for callers
 * whose device memory is owned by another allocator (a PyTorch caching
 * allocator, a serving process with a fixed memory budget) and who cannot
 * let a library call cudaMalloc/cudaFree, which take memory outside their
 * pool and, for cudaFree, synchronise the device.
 *   misfit[t] = 1/2 sum_{s < nsteps} (syn[s][t] - obs[s][t])^2, t < ntraces
 *   *total    = sum_t misfit[t]
 * syn, obs: device FP32 [nsteps][ntraces] (e.g. the [nt][2][nrec] traces of
 * one shot, ntraces = 2 nrec); residual: device FP32 [nsteps][ntraces]
 * receiving syn - obs, or NULL; misfit: host [ntraces] or NULL; total: host.
 * Work runs on `stream` (a cudaStream_t; NULL = legacy default stream) of
 * the current device, and the call returns after synchronising it.
 * Scratch: a fixed device array of SEIDART_NOALLOC_MAX_TRACES + 32 doubles
 * (64.25 KiB); ntraces above SEIDART_NOALLOC_MAX_TRACES returns
 * SEIDART_ERR_ARG with the reason in seidart_last_error().  Its ntraces
 * per-trace accumulators must start at zero: each call clears them on
 * `stream` before use.  The first call on each device looks the array up
 * (cudaGetSymbolAddress with that device current, which may load the
 * module); make that first call before any stream capture begins.  Every
 * call waits for `stream` to finish before it returns, because it copies
 * the results into host memory, so it must not be issued on a stream that
 * is being captured into a CUDA graph.  The looked-up address is kept for the life
 * of the process, so cudaDeviceReset between calls is not supported.  Calls
 * that overlap on one device share the scratch and race: serialise them. */
#define SEIDART_NOALLOC_MAX_TRACES 8192
int seidart_trace_misfit_noalloc(const float* syn, const float* obs, float* residual, int nsteps, int ntraces,
                                 double* misfit, double* total, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SEIDART_GPU_H */
