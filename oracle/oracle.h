/*
 * oracle.h -- CPU FP64 restatement of the reference CPML-FDTD time loops.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker for the GPU solvers: only
 * the tests, the smoke check and the CPU-baseline leg of the benchmark may load
 * it.  The product library never links or calls it.
 *
 * Parity status: UNPINNED.  The reference (Fortran 2008, src/fortran/*.f08)
 * ships no tests, golden vectors or fixtures, and it cannot be compiled in this
 * environment (no Fortran compiler, no json-fortran).  This file restates its
 * loops line by line; confidence comes from a second, independent numpy
 * restatement (oracle/restate_np.py) and from physics known-answer tests.
 *
 * Each oracle_* call advances `nsteps` steps numbered it0+1 .. it0+nsteps
 * (1-based like the reference's `do it = 1, time_steps`), updating `fields`
 * and the full-grid CPML memory arrays `mem` in place.  Receiver traces are
 * written as [nsteps][ncomp][nrec] (complex: interleaved re/im), norms as
 * [nsteps] (seismic3: velocity norms then, at norms + nsteps, stress norms).
 * Return value: 0, or the 1-based step at which max|v| exceeded 1e25 (the
 * reference's `stop 'code became unstable and blew up'`).
 */
#ifndef SEIDART_ORACLE_H
#define SEIDART_ORACLE_H
#include "../include/seidart_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

int oracle_seismic2(const SeidartDomain* d, const SeidartSource* s, int density_code,
                    const double* const* model, const double* const* srcfn,
                    double* const* fields, double* const* mem, int it0, int nsteps,
                    int nrec, const int* rec, double* traces, double* norms);
int oracle_seismic25(const SeidartDomain* d, const SeidartSource* s, int density_code,
                     const double* const* model, const double* const* srcfn,
                     double* const* fields, double* const* mem, int it0, int nsteps,
                     int nrec, const int* rec, double* traces, double* norms);
int oracle_seismic3(const SeidartDomain* d, const SeidartSource* s, int density_code,
                    const double* const* model, const double* const* srcfn,
                    double* const* fields, double* const* mem, int it0, int nsteps,
                    int nrec, const int* rec, double* traces, double* norms);
int oracle_electromag2(const SeidartDomain* d, const SeidartSource* s,
                       const double* const* model, const double* const* srcfn,
                       double* const* fields, double* const* mem, int it0, int nsteps,
                       int nrec, const int* rec, double* traces, double* norms);
int oracle_electromag25(const SeidartDomain* d, const SeidartSource* s,
                        const double* const* model, const double* const* srcfn,
                        double* const* fields, double* const* mem, int it0, int nsteps,
                        int nrec, const int* rec, double* traces, double* norms);
int oracle_electromag3(const SeidartDomain* d, const SeidartSource* s,
                       const double* const* model, const double* const* srcfn,
                       double* const* fields, double* const* mem, int it0, int nsteps,
                       int nrec, const int* rec, double* traces, double* norms);
/* Number of OpenMP threads the build uses (1 without OpenMP). */
int oracle_threads(void);

/* Plane-wave source for the following oracle_* calls (NULL or on = 0: point
 * sources).  v is the background speed (cbackground / vbackground) and eta
 * the impedance (EM), which the reference takes from LAPACK eigenvalues
 * (tensor_operations.f08); the caller computes them the same way.
 * p_wave: source_type "pwp" (elastic); wavelet 0 gaus0, 1 gaus1, 2 gaus2. */
typedef struct OraclePw {
    int on, p_wave, wavelet;
    double x_z_rotation, x_y_rotation, y_z_rotation, amplitude, frequency, v, eta;
} OraclePw;
void oracle_set_plane_wave(const OraclePw* pw);

#ifdef __cplusplus
}
#endif
#endif
