/*
 * oracle.c -- CPU FP64 restatement of the reference CPML-FDTD time loops.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  Parity status:
 * UNPINNED -- see oracle.h.
 *
 * The loops below follow src/fortran/cpmlfdtd.f08 of the reference statement
 * by statement: same loop bounds, same expression trees (left-to-right), same
 * quirks.  Indices are the reference's 1-based Fortran indices; IX2/IX3 map
 * them onto the 0-based column-major arrays.  Built twice from this one file:
 *   parity   : -O2 -fno-fast-math -ffp-contract=off   (bit-reproducible)
 *   baseline : -O3 -ffast-math -funroll-loops -ffp-contract=fast -fopenmp
 *              (the reference's production flags, build.sh:123, minus
 *              -march=native so the same recipe builds on x86 and Arm)
 *
 * Mixed real/complex arithmetic (seismic25, electromag25) is written out the
 * way GCC lowers gfortran's complex expressions when one operand is known to
 * be real or purely imaginary: real*complex and complex/real act on each
 * component, complex+real touches only the real part, and
 * IUNIT*ky*z = (-(ky*im z), ky*re z).
 */
#include <math.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

#define STABILITY_THRESHOLD 1.0e25
/* constants.f08:7-12 */
static const double PI_C = 3.141592653589793238462643;
#define EPS0 8.85418782e-12
#define MU0 (4.0 * PI_C * 1.0e-7)

int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* averaging.f08:5-25 */
static inline double scalar_mean(double a, double b, int code) {
    switch (code) {
    case 1: return 2.0 * a * b / (a + b);
    case 2: return sqrt(a * b);
    case 3: return 0.5 * (a + b);
    default: return a;
    }
}

#define IX2(i, k) ((size_t)((i) - 1) + (size_t)nx * (size_t)((k) - 1))
#define IX3(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))

static inline double src_at(const double* a, int it) { return a ? a[it - 1] : 0.0; }

/* =====================================================================
 * Plane-wave sources: plane_wave_source.f08 statement by statement.
 * Fortran matrices are kept column-major: A(i,j) = A[(i-1) + 3*(j-1)].
 * ===================================================================== */
static OraclePw g_pw;
static int g_pw_on = 0;
void oracle_set_plane_wave(const OraclePw* pw) {
    g_pw_on = pw && pw->on;
    if (g_pw_on) g_pw = *pw;
}

#define F3(A, i, j) (A)[((i) - 1) + 3 * ((j) - 1)]
static void matmul33(const double* A, const double* B, double* C) {
    for (int i = 1; i <= 3; ++i)
        for (int j = 1; j <= 3; ++j) {
            double acc = 0.0;
            for (int k = 1; k <= 3; ++k) acc += F3(A, i, k) * F3(B, k, j);
            F3(C, i, j) = acc;
        }
}
static void matvec3(const double* A, const double* x, double* y) {
    for (int i = 1; i <= 3; ++i) {
        double acc = 0.0;
        for (int k = 1; k <= 3; ++k) acc += F3(A, i, k) * x[k - 1];
        y[i - 1] = acc;
    }
}
static double pw_norm2(const double* v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static double pw_dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* rotmat: plane_wave_source.f08:76-108 (reshape fills columns) */
static void pw_rotmat(double axz, double axy, double ayz, double* R) {
    const double deg2rad = 3.1415926535897932384626433832795 / 180;
    const double cx = cos(deg2rad * ayz), cy = cos(deg2rad * axz), cz = cos(deg2rad * axy);
    const double sx = sin(deg2rad * ayz), sy = sin(deg2rad * axz), sz = sin(deg2rad * axy);
    const double Rx[9] = {1.0, 0.0, 0.0, 0.0, cx, -sx, 0.0, sx, cx};
    const double Ry[9] = {cy, 0.0, sy, 0.0, 1.0, 0.0, -sy, 0.0, cy};
    const double Rz[9] = {cz, -sz, 0.0, sz, cz, 0.0, 0.0, 0.0, 1.0};
    double T[9];
    matmul33(Rz, Rx, T);
    matmul33(Ry, T, R);
}

/* direction_polarization_vector: plane_wave_source.f08:110-139 */
static void pw_direction(double axz, double axy, double ayz, double* p, double* ehat) {
    const double k0[3] = {0.0, 0.0, 1.0}, e0[3] = {1.0, 0.0, 0.0};
    double R[9], tmp[3];
    pw_rotmat(axz, axy, ayz, R);
    matvec3(R, k0, p);
    double nrm = pw_norm2(p);
    if (nrm > 0.0) for (int q = 0; q < 3; ++q) p[q] = p[q] / nrm;
    matvec3(R, e0, tmp);
    double d = pw_dot(tmp, p);
    for (int q = 0; q < 3; ++q) tmp[q] = tmp[q] - d * p[q];
    nrm = pw_norm2(tmp);
    if (nrm > 0.0) {
        for (int q = 0; q < 3; ++q) ehat[q] = tmp[q] / nrm;
    } else {
        if (fabs(p[0]) < 0.9) { tmp[0] = 1.0; tmp[1] = 0.0; tmp[2] = 0.0; }
        else { tmp[0] = 0.0; tmp[1] = 1.0; tmp[2] = 0.0; }
        d = pw_dot(tmp, p);
        for (int q = 0; q < 3; ++q) tmp[q] = tmp[q] - d * p[q];
        nrm = pw_norm2(tmp);
        for (int q = 0; q < 3; ++q) ehat[q] = nrm > 0.0 ? tmp[q] / nrm : 0.0;
    }
}

/* wavelet: plane_wave_source.f08:141-161 */
static double pw_wavelet(double t, double f0, int type) {
    const double t0 = 1.5 / f0;
    const double a = 3.1415926535897932384626433832795 * f0 * (t - t0);
    const double g = exp(-a * a);
    if (type == 1) return -2.0 * a * g;
    if (type == 2) return (1.0 - 2.0 * a * a) * g;
    return g;
}

/* boundary_seismic_field: plane_wave_source.f08:196-230 */
static void pw_seismic_field(const double* r, const double* r0, double t, double* V, double* strain) {
    double p[3], ehat[3], dr[3];
    pw_direction(g_pw.x_z_rotation, g_pw.x_y_rotation, g_pw.y_z_rotation, p, ehat);
    if (g_pw.p_wave) for (int q = 0; q < 3; ++q) ehat[q] = p[q];
    for (int q = 0; q < 3; ++q) dr[q] = r[q] - r0[q];
    const double tau = t - pw_dot(p, dr) / g_pw.v;
    const double s = g_pw.amplitude * pw_wavelet(tau, g_pw.frequency, g_pw.wavelet);
    for (int q = 0; q < 3; ++q) V[q] = s * ehat[q];
    const double scale = -s / g_pw.v;
    strain[0] = scale * ehat[0] * p[0];
    strain[1] = scale * ehat[1] * p[1];
    strain[2] = scale * ehat[2] * p[2];
    strain[3] = scale * (ehat[1] * p[2] + ehat[2] * p[1]);
    strain[4] = scale * (ehat[0] * p[2] + ehat[2] * p[0]);
    strain[5] = scale * (ehat[0] * p[1] + ehat[1] * p[0]);
}

/* boundary_em_field: plane_wave_source.f08:163-194 */
static void pw_em_field(const double* r, const double* r0, double t, double* E, double* H) {
    double p[3], ehat[3], dr[3], hhat[3];
    pw_direction(g_pw.x_z_rotation, g_pw.x_y_rotation, g_pw.y_z_rotation, p, ehat);
    for (int q = 0; q < 3; ++q) dr[q] = r[q] - r0[q];
    const double tau = t - pw_dot(p, dr) / g_pw.v;
    const double s = g_pw.amplitude * pw_wavelet(tau, g_pw.frequency, g_pw.wavelet);
    for (int q = 0; q < 3; ++q) E[q] = s * ehat[q];
    hhat[0] = p[1] * ehat[2] - p[2] * ehat[1];
    hhat[1] = p[2] * ehat[0] - p[0] * ehat[2];
    hhat[2] = p[0] * ehat[1] - p[1] * ehat[0];
    const double hn = pw_norm2(hhat);
    if (hn > 0.0) for (int q = 0; q < 3; ++q) hhat[q] = hhat[q] / hn;
    for (int q = 0; q < 3; ++q) H[q] = (s / g_pw.eta) * hhat[q];
}

/* set-up of one solver (e.g. cpmlfdtd.f08:186-227): active faces, r0, the
 * face locations and the 1-based loop ranges (inset 2, electromag3: 3) */
typedef struct PwGeom {
    int active[6];
    double r0[3], loc[3];
    int imin, imax, jmin, jmax, kmin, kmax;
} PwGeom;
static void pw_geom(const SeidartDomain* d, int three, int inset, PwGeom* G) {
    double p[3], ehat[3];
    pw_direction(g_pw.x_z_rotation, g_pw.x_y_rotation, g_pw.y_z_rotation, p, ehat);
    const double eps = 1.0 * 1.0e-6;
    for (int q = 0; q < 6; ++q) G->active[q] = 0;
    if (p[0] > eps) G->active[0] = 1;
    if (p[0] < -eps) G->active[1] = 1;
    if (p[1] > eps) G->active[2] = 1;
    if (p[1] < -eps) G->active[3] = 1;
    if (p[2] > eps) G->active[4] = 1;
    if (p[2] < -eps) G->active[5] = 1;
    const double XMIN = d->dx * (1 + d->cpml), XMAX = d->dx * (d->nx - d->cpml);
    const double YMIN = d->dy * (1 + d->cpml), YMAX = d->dy * (d->ny - d->cpml);
    const double ZMIN = d->dz * (1 + d->cpml), ZMAX = d->dz * (d->nz - d->cpml);
    const double XMID = 0.50 * (XMIN + XMAX), YMID = 0.50 * (YMIN + YMAX), ZMID = 0.50 * (ZMIN + ZMAX);
    G->r0[0] = XMID; G->r0[1] = three ? YMID : 0.0; G->r0[2] = ZMID;
    G->loc[0] = XMID; G->loc[1] = YMID; G->loc[2] = ZMID;
    if (G->active[0]) { G->r0[0] = XMIN; G->loc[0] = XMIN; }
    if (G->active[1]) { G->r0[0] = XMAX; G->loc[0] = XMAX; }
    if (three && G->active[2]) { G->r0[1] = YMIN; G->loc[1] = YMIN; }
    if (three && G->active[3]) { G->r0[1] = YMAX; G->loc[1] = YMAX; }
    if (G->active[4]) { G->r0[2] = ZMIN; G->loc[2] = ZMIN; }
    if (G->active[5]) { G->r0[2] = ZMAX; G->loc[2] = ZMAX; }
    G->imin = d->cpml + inset; G->imax = d->nx - d->cpml - (inset - 1);
    G->jmin = d->cpml + inset; G->jmax = d->ny - d->cpml - (inset - 1);
    G->kmin = d->cpml + inset; G->kmax = d->nz - d->cpml - (inset - 1);
}
static int nint_(double x) { return (int)lround(x); }

/* C_ij (1-based Voigt row a, column b) of the upper-triangle C21 order */
static double cij(const double* const* C, int a, int b, size_t c) {
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    return C[(lo - 1) * 6 - (lo - 1) * (lo - 2) / 2 + (hi - lo)][c];
}
/* add_plane_wave_stress: cpmlfdtd.f08:16-50 (s[0..5] = sxx syy szz syz sxz sxy) */
static void pw_add_stress(const double* const* C, size_t c, const double* st, double* s) {
    for (int a = 1; a <= 6; ++a) {
        double acc = s[a - 1];
        for (int b = 1; b <= 6; ++b) acc = acc + cij(C, a, b, c) * st[b - 1];
        s[a - 1] = acc;
    }
}
/* 3D face loops of seismic3 / electromag3 (x face, y face, z face), calling
 * body(cell, r) for every cell of each active face in the reference's order */
#define PW_FACES3(G, dx, dy, dz, ...)                                                             \
    do {                                                                                          \
        double r[3];                                                                              \
        if ((G).active[0] || (G).active[1]) {                                                     \
            const int ii = nint_((G).loc[0] / (dx));                                              \
            for (int jj = (G).jmin; jj <= (G).jmax; ++jj)                                         \
                for (int kk = (G).kmin; kk <= (G).kmax; ++kk) {                                   \
                    r[0] = (G).loc[0]; r[1] = jj * (dy); r[2] = kk * (dz);                        \
                    const size_t c = IX3(ii, jj, kk);                                             \
                    __VA_ARGS__                                                                   \
                }                                                                                 \
        }                                                                                         \
        if ((G).active[2] || (G).active[3]) {                                                     \
            const int jj = nint_((G).loc[1] / (dy));                                              \
            for (int ii = (G).imin; ii <= (G).imax; ++ii)                                         \
                for (int kk = (G).kmin; kk <= (G).kmax; ++kk) {                                   \
                    r[0] = ii * (dx); r[1] = (G).loc[1]; r[2] = kk * (dz);                        \
                    const size_t c = IX3(ii, jj, kk);                                             \
                    __VA_ARGS__                                                                   \
                }                                                                                 \
        }                                                                                         \
        if ((G).active[4] || (G).active[5]) {                                                     \
            const int kk = nint_((G).loc[2] / (dz));                                              \
            for (int ii = (G).imin; ii <= (G).imax; ++ii)                                         \
                for (int jj = (G).jmin; jj <= (G).jmax; ++jj) {                                   \
                    r[0] = ii * (dx); r[1] = jj * (dy); r[2] = (G).loc[2];                        \
                    const size_t c = IX3(ii, jj, kk);                                             \
                    __VA_ARGS__                                                                   \
                }                                                                                 \
        }                                                                                         \
    } while (0)

/* =====================================================================
 * seismic2: cpmlfdtd.f08:311-576
 * ===================================================================== */
int oracle_seismic2(const SeidartDomain* d, const SeidartSource* s, int density_code,
                    const double* const* model, const double* const* srcfn,
                    double* const* fields, double* const* mem, int it0, int nsteps,
                    int nrec, const int* rec, double* traces, double* norms) {
    const int nx = d->nx, nz = d->nz;
    const double dx = d->dx, dz = d->dz, dt = s->dt;
    const double *c11 = model[S2_C11], *c13 = model[S2_C13], *c15 = model[S2_C15],
                 *c33 = model[S2_C33], *c35 = model[S2_C35], *c55 = model[S2_C55],
                 *rho = model[S2_RHO], *gamma_x = model[S2_GX], *gamma_z = model[S2_GZ],
                 *gamma_xz = model[S2_GXZ], *kappa = model[S2_KAPPA],
                 *kappa_half = model[S2_KAPPAH], *acoef = model[S2_ACOEF],
                 *acoef_half = model[S2_ACOEFH], *bcoef = model[S2_BCOEF],
                 *bcoef_half = model[S2_BCOEFH];
    double *vx = fields[S2_VX], *vz = fields[S2_VZ], *sigmaxx = fields[S2_SXX],
           *sigmazz = fields[S2_SZZ], *sigmaxz = fields[S2_SXZ];
    double *m_dvx_dx1 = mem[S2_M_DVX_DX1], *m_dvx_dz1 = mem[S2_M_DVX_DZ1],
           *m_dvz_dx1 = mem[S2_M_DVZ_DX1], *m_dvz_dz1 = mem[S2_M_DVZ_DZ1],
           *m_dvx_dx2 = mem[S2_M_DVX_DX2], *m_dvx_dz2 = mem[S2_M_DVX_DZ2],
           *m_dvz_dx2 = mem[S2_M_DVZ_DX2], *m_dvz_dz2 = mem[S2_M_DVZ_DZ2],
           *m_dsxx_dx = mem[S2_M_DSXX_DX], *m_dszz_dz = mem[S2_M_DSZZ_DZ],
           *m_dsxz_dx = mem[S2_M_DSXZ_DX], *m_dsxz_dz = mem[S2_M_DSXZ_DZ];
    const int isource = s->xind + d->cpml, jsource = s->zind + d->cpml;

    for (int step = 0; step < nsteps; ++step) {
        const int it = it0 + step + 1;
        /* stress, normal components: cpmlfdtd.f08:324-353 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int j = 3; j <= nz - 1; ++j)
            for (int i = 2; i <= nx - 2; ++i) {
                const size_t c = IX2(i, j);
                double dvx_dx = (27.0 * (vx[IX2(i + 1, j)] - vx[c]) - (vx[IX2(i + 2, j)] - vx[IX2(i - 1, j)])) / (24.0 * dx);
                double dvz_dz = (27.0 * (vz[c] - vz[IX2(i, j - 1)]) - (vz[IX2(i, j + 1)] - vz[IX2(i, j - 2)])) / (24.0 * dz);
                double dvz_dx = (27.0 * (vz[IX2(i + 1, j)] - vz[c]) - (vz[IX2(i + 2, j)] - vz[IX2(i - 1, j)])) / (24.0 * dx);
                double dvx_dz = (27.0 * (vx[c] - vx[IX2(i, j - 1)]) - (vx[IX2(i, j + 1)] - vx[IX2(i, j - 2)])) / (24.0 * dz);
                m_dvx_dx1[c] = bcoef_half[c] * m_dvx_dx1[c] + acoef_half[c] * dvx_dx;
                m_dvx_dz1[c] = bcoef_half[c] * m_dvx_dz1[c] + acoef_half[c] * dvx_dz;
                m_dvz_dz1[c] = bcoef[c] * m_dvz_dz1[c] + acoef[c] * dvz_dz;
                m_dvz_dx1[c] = bcoef[c] * m_dvz_dx1[c] + acoef[c] * dvz_dx;
                dvx_dx = dvx_dx / kappa_half[c] + m_dvx_dx1[c];
                dvx_dz = dvx_dz / kappa_half[c] + m_dvx_dz1[c];
                dvz_dz = dvz_dz / kappa[c] + m_dvz_dz1[c];
                dvz_dx = dvz_dx / kappa[c] + m_dvz_dx1[c];
                sigmaxx[c] = (sigmaxx[c] + (c11[c] * dvx_dx + c13[c] * dvz_dz + c15[c] * (dvz_dx + dvx_dz)) * dt) /
                             (1.0 + gamma_x[c] * dt);
                sigmazz[c] = (sigmazz[c] + (c13[c] * dvx_dx + c33[c] * dvz_dz + c35[c] * (dvz_dx + dvx_dz)) * dt) /
                             (1.0 + gamma_z[c] * dt);
            }
        /* stress, shear component: cpmlfdtd.f08:362-386 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int j = 2; j <= nz - 2; ++j)
            for (int i = 3; i <= nx - 1; ++i) {
                const size_t c = IX2(i, j);
                double dvx_dx = (27.0 * (vx[c] - vx[IX2(i - 1, j)]) - (vx[IX2(i + 1, j)] - vx[IX2(i - 2, j)])) / (24.0 * dx);
                double dvz_dz = (27.0 * (vz[IX2(i, j + 1)] - vz[c]) - (vz[IX2(i, j + 2)] - vz[IX2(i, j - 1)])) / (24.0 * dz);
                double dvz_dx = (27.0 * (vz[c] - vz[IX2(i - 1, j)]) - (vz[IX2(i + 1, j)] - vz[IX2(i - 2, j)])) / (24.0 * dx);
                double dvx_dz = (27.0 * (vx[IX2(i, j + 1)] - vx[c]) - (vx[IX2(i, j + 2)] - vx[IX2(i, j - 1)])) / (24.0 * dz);
                m_dvx_dx2[c] = bcoef_half[c] * m_dvx_dx2[c] + acoef_half[c] * dvx_dx;
                m_dvx_dz2[c] = bcoef_half[c] * m_dvx_dz2[c] + acoef_half[c] * dvx_dz;
                m_dvz_dz2[c] = bcoef_half[c] * m_dvz_dz2[c] + acoef_half[c] * dvz_dz;
                m_dvz_dx2[c] = bcoef_half[c] * m_dvz_dx2[c] + acoef_half[c] * dvz_dx;
                dvx_dx = dvx_dx / kappa_half[c] + m_dvx_dx2[c];
                dvx_dz = dvx_dz / kappa_half[c] + m_dvx_dz2[c];
                dvz_dz = dvz_dz / kappa_half[c] + m_dvz_dz2[c];
                dvz_dx = dvz_dx / kappa_half[c] + m_dvz_dx2[c];
                sigmaxz[c] = (sigmaxz[c] + (c15[c] * dvx_dx + c35[c] * dvz_dz + c55[c] * (dvz_dx + dvx_dz)) * dt) /
                             (1.0 + gamma_xz[c] * dt);
            }
        /* vx: cpmlfdtd.f08:399-416 (three-term x and z stencils, reference quirk) */
#pragma omp parallel for collapse(2) schedule(static)
        for (int j = 3; j <= nz - 1; ++j)
            for (int i = 3; i <= nx - 1; ++i) {
                const size_t c = IX2(i, j);
                const double rhoxx = scalar_mean(rho[c], rho[IX2(i - 1, j)], density_code);
                const double rhozx = scalar_mean(rho[c], rho[IX2(i, j - 1)], density_code);
                double dsxx_dx = (27.0 * sigmaxx[c] - 27.0 * sigmaxx[IX2(i - 1, j)] + sigmaxx[IX2(i - 2, j)]) / (24.0 * dx);
                double dsxz_dz = (27.0 * sigmaxz[c] - 27.0 * sigmaxz[IX2(i, j - 1)] + sigmaxz[IX2(i, j - 2)]) / (24.0 * dz);
                m_dsxx_dx[c] = bcoef[c] * m_dsxx_dx[c] + acoef[c] * dsxx_dx;
                m_dsxz_dz[c] = bcoef[c] * m_dsxz_dz[c] + acoef[c] * dsxz_dz;
                dsxx_dx = dsxx_dx / kappa[c] + m_dsxx_dx[c];
                dsxz_dz = dsxz_dz / kappa[c] + m_dsxz_dz[c];
                vx[c] = vx[c] + dt * (dsxx_dx / rhoxx + dsxz_dz / rhozx);
            }
        /* vz: cpmlfdtd.f08:428-446 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int j = 2; j <= nz - 2; ++j)
            for (int i = 2; i <= nx - 2; ++i) {
                const size_t c = IX2(i, j);
                const double rhoxz = scalar_mean(rho[c], rho[IX2(i + 1, j)], density_code);
                const double rhozz = scalar_mean(rho[c], rho[IX2(i, j + 1)], density_code);
                double dsxz_dx = (-27.0 * sigmaxz[c] + 27.0 * sigmaxz[IX2(i + 1, j)] - sigmaxz[IX2(i + 2, j)]) / (24.0 * dx);
                double dszz_dz = (-27.0 * sigmazz[c] + 27.0 * sigmazz[IX2(i, j + 1)] - sigmazz[IX2(i, j + 2)]) / (24.0 * dz);
                m_dsxz_dx[c] = bcoef_half[c] * m_dsxz_dx[c] + acoef_half[c] * dsxz_dx;
                m_dszz_dz[c] = bcoef_half[c] * m_dszz_dz[c] + acoef_half[c] * dszz_dz;
                dsxz_dx = dsxz_dx / kappa_half[c] + m_dsxz_dx[c];
                dszz_dz = dszz_dz / kappa_half[c] + m_dszz_dz[c];
                vz[c] = vz[c] + dt * (dsxz_dx / rhoxz + dszz_dz / rhozz);
            }
        if (g_pw_on) {  /* plane wave: cpmlfdtd.f08:454-512 */
            PwGeom G;
            pw_geom(d, 0, 2, &G);
            const double t = it * s->dt;
            double r[3], V[3], st[6];
            for (int face = 0; face < 2; ++face) {
                const int xface = face == 0;
                if (xface ? !(G.active[0] || G.active[1]) : !(G.active[4] || G.active[5])) continue;
                const int fixed = xface ? nint_(G.loc[0] / dx) : nint_(G.loc[2] / dz);
                const int lo = xface ? G.kmin : G.imin, hi = xface ? G.kmax : G.imax;
                for (int ip = lo; ip <= hi; ++ip) {
                    if (xface) { r[0] = G.loc[0]; r[1] = 0.0; r[2] = ip * dz; }
                    else { r[0] = ip * dx; r[1] = 0.0; r[2] = G.loc[2]; }
                    pw_seismic_field(r, G.r0, t, V, st);
                    const size_t c = xface ? IX2(fixed, ip) : IX2(ip, fixed);
                    vx[c] = vx[c] + V[0];
                    vz[c] = vz[c] + V[2];
                    sigmaxx[c] = sigmaxx[c] + c11[c] * st[0] + c13[c] * st[2] + c15[c] * st[4];
                    sigmazz[c] = sigmazz[c] + c13[c] * st[0] + c33[c] * st[2] + c35[c] * st[4];
                    sigmaxz[c] = sigmaxz[c] + c15[c] * st[0] + c35[c] * st[2] + c55[c] * st[4];
                }
            }
        } else
        /* point source: cpmlfdtd.f08:519-523 (no dt on the force terms) */
        {
            const size_t c = IX2(isource, jsource), c1 = IX2(isource + 1, jsource + 1);
            sigmaxx[c] = sigmaxx[c] + src_at(srcfn[S2_SRCXX], it) / rho[c];
            sigmaxz[c1] = sigmaxz[c1] + src_at(srcfn[S2_SRCXZ], it) / rho[c1];
            sigmazz[c] = sigmazz[c] + src_at(srcfn[S2_SRCZZ], it) / rho[c];
            vx[c] = vx[c] + src_at(srcfn[S2_SRCX], it) / rho[c];
            vz[c] = vz[c] + src_at(srcfn[S2_SRCZ], it) / rho[c];
        }
        /* Dirichlet edges: cpmlfdtd.f08:534-549 */
        for (int j = 1; j <= nz; ++j) {
            vx[IX2(1, j)] = 0.0; vx[IX2(nx, j)] = 0.0;
            vz[IX2(1, j)] = 0.0; vz[IX2(nx, j)] = 0.0;
        }
        for (int i = 1; i <= nx; ++i) {
            vx[IX2(i, 1)] = 0.0; vx[IX2(i, nz)] = 0.0;
            vz[IX2(i, 1)] = 0.0; vz[IX2(i, nz)] = 0.0;
        }
        /* max-norm: cpmlfdtd.f08:552-567 */
        double velocnorm = 0.0;
#pragma omp parallel for collapse(2) reduction(max : velocnorm) schedule(static)
        for (int j = 1; j <= nz; ++j)
            for (int i = 1; i <= nx; ++i) {
                const size_t c = IX2(i, j);
                const double n = sqrt(vx[c] * vx[c] + vz[c] * vz[c]);
                velocnorm = velocnorm > n ? velocnorm : n;
            }
        if (norms) norms[step] = velocnorm;
        if (traces)
            for (int r = 0; r < nrec; ++r) {
                traces[((size_t)step * 2 + 0) * nrec + r] = vx[rec[r]];
                traces[((size_t)step * 2 + 1) * nrec + r] = vz[rec[r]];
            }
        if (velocnorm > STABILITY_THRESHOLD) return it;
    }
    return 0;
}

/* =====================================================================
 * complex helpers for the 2.5D solvers (interleaved re/im arrays)
 * ===================================================================== */
typedef struct { double re, im; } cplx;
static inline cplx cld(const double* a, size_t c) { cplx z = {a[2 * c], a[2 * c + 1]}; return z; }
static inline void cst(double* a, size_t c, cplx z) { a[2 * c] = z.re; a[2 * c + 1] = z.im; }
static inline cplx cadd(cplx a, cplx b) { cplx z = {a.re + b.re, a.im + b.im}; return z; }
static inline cplx csub(cplx a, cplx b) { cplx z = {a.re - b.re, a.im - b.im}; return z; }
static inline cplx crmul(double r, cplx a) { cplx z = {r * a.re, r * a.im}; return z; }
static inline cplx cmulr(cplx a, double r) { cplx z = {a.re * r, a.im * r}; return z; }
static inline cplx cdivr(cplx a, double r) { cplx z = {a.re / r, a.im / r}; return z; }
static inline cplx cneg(cplx a) { cplx z = {-a.re, -a.im}; return z; }
/* IUNIT * ky * z */
static inline cplx ciky(double ky, cplx a) { cplx z = {-(ky * a.im), ky * a.re}; return z; }

/* (27(f[p1]-f[p0]) - (f[p2]-f[m1])) / (24 h) */
static inline cplx cd4(const double* f, size_t p1, size_t p0, size_t p2, size_t m1, double h24) {
    return cdivr(csub(crmul(27.0, csub(cld(f, p1), cld(f, p0))), csub(cld(f, p2), cld(f, m1))), h24);
}
/* m = b*m + a*d ; returns d/k + m */
static inline cplx ccpml(double* m, size_t c, double b, double a, double k, cplx dv) {
    cplx mv = cadd(crmul(b, cld(m, c)), crmul(a, dv));
    cst(m, c, mv);
    return cadd(cdivr(dv, k), mv);
}

/* array_averaging2d (averaging.f08:27-80): in-place, ascending loops, so '+i'
 * and '+j' produce running averages (each value mixes the updated neighbour). */
static void array_averaging2d(double* a, int ni, int nj, int code, int dir) {
    /* dir: 0 '+i', 1 '-i', 2 '+j', 3 '-j' */
    const int nx = ni;
    switch (dir) {
    case 0: for (int j = 1; j <= nj; ++j) for (int i = 2; i <= ni; ++i) a[IX2(i, j)] = scalar_mean(a[IX2(i, j)], a[IX2(i - 1, j)], code); break;
    case 1: for (int j = 1; j <= nj; ++j) for (int i = 1; i <= ni - 1; ++i) a[IX2(i, j)] = scalar_mean(a[IX2(i, j)], a[IX2(i + 1, j)], code); break;
    case 2: for (int j = 2; j <= nj; ++j) for (int i = 1; i <= ni; ++i) a[IX2(i, j)] = scalar_mean(a[IX2(i, j)], a[IX2(i, j - 1)], code); break;
    default: for (int j = 1; j <= nj - 1; ++j) for (int i = 1; i <= ni; ++i) a[IX2(i, j)] = scalar_mean(a[IX2(i, j)], a[IX2(i, j + 1)], code); break;
    }
}

#include <stdlib.h>

/* =====================================================================
 * seismic25: cpmlfdtd.f08:931-1313 (complex fields, d/dy = i ky)
 * ===================================================================== */
int oracle_seismic25(const SeidartDomain* d, const SeidartSource* s, int density_code,
                     const double* const* model, const double* const* srcfn,
                     double* const* fields, double* const* mem, int it0, int nsteps,
                     int nrec, const int* rec, double* traces, double* norms) {
    const int nx = d->nx, nz = d->nz;
    const double dx = d->dx, dz = d->dz, dt = s->dt, ky = s->ky;
    const double* C[21];
    for (int q = 0; q < 21; ++q) C[q] = model[q];
#define CC(q) C[SEIDART_##q][c]
    const double *rho = model[SEIDART_RHO3], *gamma_x = model[SEIDART_GX3],
                 *gamma_y = model[SEIDART_GY3], *gamma_z = model[SEIDART_GZ3],
                 *gamma_xy = model[SEIDART_GXY3], *gamma_yz = model[SEIDART_GYZ3],
                 *gamma_xz = model[SEIDART_GXZ3], *kappa = model[SEIDART_KAPPA3],
                 *kappa_half = model[SEIDART_KAPPAH3], *acoef = model[SEIDART_ACOEF3],
                 *acoef_half = model[SEIDART_ACOEFH3], *bcoef = model[SEIDART_BCOEF3],
                 *bcoef_half = model[SEIDART_BCOEFH3];
    double *vx = fields[S3_VX], *vy = fields[S3_VY], *vz = fields[S3_VZ],
           *sxx = fields[S3_SXX], *sxy = fields[S3_SXY], *sxz = fields[S3_SXZ],
           *syy = fields[S3_SYY], *syz = fields[S3_SYZ], *szz = fields[S3_SZZ];
    const int isource = s->xind + d->cpml, ksource = s->zind + d->cpml;
    const size_t N = (size_t)nx * nz;

    /* density averaging: cpmlfdtd.f08:889-898 */
    double* rr = (double*)malloc(sizeof(double) * N * 6);
    if (!rr) return -1;
    double *rhoxx = rr, *rhozx = rr + N, *rhoxy = rr + 2 * N, *rhozy = rr + 3 * N,
           *rhoxz = rr + 4 * N, *rhozz = rr + 5 * N;
    const double *rhoyx = rho, *rhoyy = rho, *rhoyz = rho;
    for (int q = 0; q < 6; ++q) memcpy(rr + q * N, rho, sizeof(double) * N);
    array_averaging2d(rhoxx, nx, nz, density_code, 0);
    array_averaging2d(rhozx, nx, nz, density_code, 2);
    array_averaging2d(rhoxy, nx, nz, density_code, 1);
    array_averaging2d(rhozy, nx, nz, density_code, 2);
    array_averaging2d(rhoxz, nx, nz, density_code, 1);
    array_averaging2d(rhozz, nx, nz, density_code, 3);

    const double h24x = 24.0 * dx, h24z = 24.0 * dz;
    int status = 0;
    for (int step = 0; step < nsteps; ++step) {
        const int it = it0 + step + 1;
        /* the four stress loops share this body; L selects stencils and
         * coefficients (cpmlfdtd.f08:941-1117) */
        for (int L = 1; L <= 4; ++L) {
            const int klo = (L <= 2) ? 3 : 2, khi = (L <= 2) ? nz - 1 : nz - 2;
            const int ilo = (L == 1 || L == 4) ? 2 : 3, ihi = (L == 1 || L == 4) ? nx - 2 : nx - 1;
            const int xfwd = (L == 1 || L == 4), zfwd = (L >= 3);
            /* CPML coefficient choice per loop: x then z (full = 0, half = 1) */
            const int xhalf = (L == 1 || L == 4), zhalf = (L != 1);
            double* const* M = mem + 6 * (L - 1);
#pragma omp parallel for collapse(2) schedule(static)
            for (int k = klo; k <= khi; ++k)
                for (int i = ilo; i <= ihi; ++i) {
                    const size_t c = IX2(i, k);
                    cplx dvdx[3], dvdy[3], dvdz[3];
                    const double* v[3] = {vx, vy, vz};
                    for (int q = 0; q < 3; ++q) {
                        if (xfwd) dvdx[q] = cd4(v[q], IX2(i + 1, k), c, IX2(i + 2, k), IX2(i - 1, k), h24x);
                        else dvdx[q] = cd4(v[q], c, IX2(i - 1, k), IX2(i + 1, k), IX2(i - 2, k), h24x);
                        dvdy[q] = ciky(ky, cld(v[q], c));
                        if (zfwd) dvdz[q] = cd4(v[q], IX2(i, k + 1), c, IX2(i, k + 2), IX2(i, k - 1), h24z);
                        else dvdz[q] = cd4(v[q], c, IX2(i, k - 1), IX2(i, k + 1), IX2(i, k - 2), h24z);
                    }
                    const double bx = xhalf ? bcoef_half[c] : bcoef[c], ax = xhalf ? acoef_half[c] : acoef[c],
                                 kx = xhalf ? kappa_half[c] : kappa[c];
                    const double bz = zhalf ? bcoef_half[c] : bcoef[c], az = zhalf ? acoef_half[c] : acoef[c],
                                 kz = zhalf ? kappa_half[c] : kappa[c];
                    for (int q = 0; q < 3; ++q) dvdx[q] = ccpml(M[q], c, bx, ax, kx, dvdx[q]);
                    for (int q = 0; q < 3; ++q) dvdz[q] = ccpml(M[3 + q], c, bz, az, kz, dvdz[q]);
                    const cplx dvx_dx = dvdx[0], dvy_dx = dvdx[1], dvz_dx = dvdx[2];
                    const cplx dvx_dy = dvdy[0], dvy_dy = dvdy[1], dvz_dy = dvdy[2];
                    const cplx dvx_dz = dvdz[0], dvy_dz = dvdz[1], dvz_dz = dvdz[2];
                    const cplx e4 = cadd(dvy_dz, dvz_dy), e5 = cadd(dvx_dz, dvz_dx), e6 = cadd(dvy_dx, dvx_dy);
#define STRESS25(arr, a1, a2, a3, a4, a5, a6, g)                                                             \
    cst(arr, c, cdivr(cadd(cld(arr, c),                                                                      \
                           cmulr(cadd(cadd(cadd(cadd(cadd(crmul(CC(a1), dvx_dx), crmul(CC(a2), dvy_dy)),     \
                                                     crmul(CC(a3), dvz_dz)), crmul(CC(a4), e4)),             \
                                           crmul(CC(a5), e5)), crmul(CC(a6), e6)), dt)),                     \
                      1.0 + (g)[c] * dt))
                    if (L == 1) {
                        STRESS25(sxx, C11, C12, C13, C14, C15, C16, gamma_x);
                        STRESS25(syy, C12, C22, C23, C24, C25, C26, gamma_y);
                        STRESS25(szz, C13, C23, C33, C34, C35, C36, gamma_z);
                    } else if (L == 2) {
                        STRESS25(sxy, C16, C26, C36, C46, C56, C66, gamma_xy);
                    } else if (L == 3) {
                        STRESS25(sxz, C15, C25, C35, C45, C55, C56, gamma_xz);
                    } else {
                        STRESS25(syz, C14, C24, C34, C44, C45, C46, gamma_yz);
                    }
#undef STRESS25
                }
        }
        /* vx: cpmlfdtd.f08:1130-1146 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 3; k <= nz - 1; ++k)
            for (int i = 3; i <= nx - 1; ++i) {
                const size_t c = IX2(i, k);
                cplx a = cdivr(cadd(csub(crmul(27.0, cld(sxx, c)), crmul(27.0, cld(sxx, IX2(i - 1, k)))), cld(sxx, IX2(i - 2, k))), h24x);
                cplx b = ciky(ky, cld(sxy, c));
                cplx e = cdivr(cadd(csub(crmul(27.0, cld(sxz, c)), crmul(27.0, cld(sxz, IX2(i, k - 1)))), cld(sxz, IX2(i, k - 2))), h24z);
                a = ccpml(mem[S25_M_DSXX_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], a);
                e = ccpml(mem[S25_M_DSXZ_DZ], c, bcoef_half[c], acoef_half[c], kappa_half[c], e);
                cst(vx, c, cadd(cld(vx, c), cmulr(cadd(cadd(cdivr(a, rhoxx[c]), cdivr(b, rhoyx[c])), cdivr(e, rhozx[c])), dt)));
            }
        /* vy: cpmlfdtd.f08:1158-1174 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 3; k <= nz - 1; ++k)
            for (int i = 2; i <= nx - 2; ++i) {
                const size_t c = IX2(i, k);
                cplx a = cdivr(csub(cadd(cneg(crmul(27.0, cld(sxy, c))), crmul(27.0, cld(sxy, IX2(i + 1, k)))), cld(sxy, IX2(i + 2, k))), h24x);
                cplx b = ciky(ky, cld(syy, c));
                cplx e = cdivr(cadd(csub(crmul(27.0, cld(syz, c)), crmul(27.0, cld(syz, IX2(i, k - 1)))), cld(syz, IX2(i, k - 2))), h24z);
                a = ccpml(mem[S25_M_DSXY_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], a);
                e = ccpml(mem[S25_M_DSYZ_DZ], c, bcoef[c], acoef[c], kappa[c], e);
                cst(vy, c, cadd(cld(vy, c), cmulr(cadd(cadd(cdivr(a, rhoxy[c]), cdivr(b, rhoyy[c])), cdivr(e, rhozy[c])), dt)));
            }
        /* vz: cpmlfdtd.f08:1186-1202 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 2; k <= nz - 2; ++k)
            for (int i = 2; i <= nx - 2; ++i) {
                const size_t c = IX2(i, k);
                cplx a = cdivr(csub(cadd(cneg(crmul(27.0, cld(sxz, c))), crmul(27.0, cld(sxz, IX2(i + 1, k)))), cld(sxz, IX2(i + 2, k))), h24x);
                cplx b = ciky(ky, cld(syz, c));
                cplx e = cdivr(csub(cadd(cneg(crmul(27.0, cld(szz, c))), crmul(27.0, cld(szz, IX2(i, k + 1)))), cld(szz, IX2(i, k + 2))), h24z);
                a = ccpml(mem[S25_M_DSXZ_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], a);
                e = ccpml(mem[S25_M_DSZZ_DZ], c, bcoef_half[c], acoef_half[c], kappa_half[c], e);
                cst(vz, c, cadd(cld(vz, c), cmulr(cadd(cadd(cdivr(a, rhoxz[c]), cdivr(b, rhoyz[c])), cdivr(e, rhozz[c])), dt)));
            }
        if (g_pw_on) {  /* plane wave: cpmlfdtd.f08:1208-1260 (real parts) */
            PwGeom G;
            pw_geom(d, 0, 2, &G);
            const double t = it * dt;
            double r[3], V[3], st[6];
            for (int face = 0; face < 2; ++face) {
                const int xface = face == 0;
                if (xface ? !(G.active[0] || G.active[1]) : !(G.active[4] || G.active[5])) continue;
                const int fixed = xface ? nint_(G.loc[0] / dx) : nint_(G.loc[2] / dz);
                const int lo = xface ? G.kmin : G.imin, hi = xface ? G.kmax : G.imax;
                for (int ip = lo; ip <= hi; ++ip) {
                    if (xface) { r[0] = G.loc[0]; r[1] = 0.0; r[2] = ip * dz; }
                    else { r[0] = ip * dx; r[1] = 0.0; r[2] = G.loc[2]; }
                    pw_seismic_field(r, G.r0, t, V, st);
                    const size_t c = xface ? IX2(fixed, ip) : IX2(ip, fixed);
                    vx[2 * c] = vx[2 * c] + V[0];
                    vy[2 * c] = vy[2 * c] + V[1];
                    vz[2 * c] = vz[2 * c] + V[2];
                    double tmp[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                    pw_add_stress(C, c, st, tmp);
                    sxx[2 * c] = sxx[2 * c] + tmp[0];
                    syy[2 * c] = syy[2 * c] + tmp[1];
                    szz[2 * c] = szz[2 * c] + tmp[2];
                    syz[2 * c] = syz[2 * c] + tmp[3];
                    sxz[2 * c] = sxz[2 * c] + tmp[4];
                    sxy[2 * c] = sxy[2 * c] + tmp[5];
                }
            }
        } else
        /* point source: cpmlfdtd.f08:1268-1276 (real part only) */
        {
#define ADDRE(arr, i, k, val) arr[2 * IX2(i, k)] = arr[2 * IX2(i, k)] + (val)
            const int is = isource, ks = ksource;
            ADDRE(sxx, is, ks, src_at(srcfn[S3_SRCXX], it) / rho[IX2(is, ks)]);
            ADDRE(sxy, is + 1, ks, src_at(srcfn[S3_SRCXY], it) / rho[IX2(is + 1, ks)]);
            ADDRE(sxz, is + 1, ks + 1, src_at(srcfn[S3_SRCXZ], it) / rho[IX2(is + 1, ks)]);
            ADDRE(syy, is, ks, src_at(srcfn[S3_SRCYY], it) / rho[IX2(is, ks)]);
            ADDRE(syz, is, ks + 1, src_at(srcfn[S3_SRCYZ], it) / rho[IX2(is, ks + 1)]);
            ADDRE(szz, is, ks, src_at(srcfn[S3_SRCZZ], it) / rho[IX2(is, ks)]);
            ADDRE(vx, is + 1, ks, src_at(srcfn[S3_SRCX], it) * dt / rho[IX2(is + 1, ks)]);
            ADDRE(vy, is, ks, src_at(srcfn[S3_SRCY], it) * dt / rho[IX2(is, ks)]);
            ADDRE(vz, is, ks + 1, src_at(srcfn[S3_SRCZ], it) * dt / rho[IX2(is, ks + 1)]);
#undef ADDRE
        }
        /* Dirichlet: cpmlfdtd.f08:1280-1285 */
        {
            double* vv[3] = {vx, vy, vz};
            for (int q = 0; q < 3; ++q) {
                for (int k = 1; k <= nz; ++k) {
                    vv[q][2 * IX2(1, k)] = vv[q][2 * IX2(1, k) + 1] = 0.0;
                    vv[q][2 * IX2(nx, k)] = vv[q][2 * IX2(nx, k) + 1] = 0.0;
                }
                for (int i = 1; i <= nx; ++i) {
                    vv[q][2 * IX2(i, 1)] = vv[q][2 * IX2(i, 1) + 1] = 0.0;
                    vv[q][2 * IX2(i, nz)] = vv[q][2 * IX2(i, nz) + 1] = 0.0;
                }
            }
        }
        /* norm: cpmlfdtd.f08:1291-1292 */
        double velocnorm = 0.0;
#pragma omp parallel for reduction(max : velocnorm) schedule(static)
        for (size_t c = 0; c < N; ++c) {
            const double a = vx[2 * c] * vx[2 * c] + vx[2 * c + 1] * vx[2 * c + 1];
            const double b = vy[2 * c] * vy[2 * c] + vy[2 * c + 1] * vy[2 * c + 1];
            const double e = vz[2 * c] * vz[2 * c] + vz[2 * c + 1] * vz[2 * c + 1];
            const double n = sqrt(a + b + e);
            velocnorm = velocnorm > n ? velocnorm : n;
        }
        if (norms) norms[step] = velocnorm;
        if (traces)
            for (int r = 0; r < nrec; ++r) {
                const double* vv[3] = {vx, vy, vz};
                for (int q = 0; q < 3; ++q) {
                    traces[2 * (((size_t)step * 3 + q) * nrec + r)] = vv[q][2 * (size_t)rec[r]];
                    traces[2 * (((size_t)step * 3 + q) * nrec + r) + 1] = vv[q][2 * (size_t)rec[r] + 1];
                }
            }
        if (velocnorm > STABILITY_THRESHOLD) { status = it; break; }
    }
#undef CC
    free(rr);
    return status;
}

/* =====================================================================
 * seismic3: cpmlfdtd.f08:1747-2277
 * ===================================================================== */
static inline double d4(const double* f, size_t p1, size_t p0, size_t p2, size_t m1, double h24) {
    return (27.0 * (f[p1] - f[p0]) - (f[p2] - f[m1])) / h24;
}
static inline double rcpml(double* m, size_t c, double b, double a, double k, double dv) {
    m[c] = b * m[c] + a * dv;
    return dv / k + m[c];
}

int oracle_seismic3(const SeidartDomain* d, const SeidartSource* s, int density_code,
                    const double* const* model, const double* const* srcfn,
                    double* const* fields, double* const* mem, int it0, int nsteps,
                    int nrec, const int* rec, double* traces, double* norms) {
    const int nx = d->nx, ny = d->ny, nz = d->nz;
    const double dx = d->dx, dy = d->dy, dz = d->dz, dt = s->dt;
    const double* C[21];
    for (int q = 0; q < 21; ++q) C[q] = model[q];
#define CC(q) C[SEIDART_##q][c]
    const double *rho = model[SEIDART_RHO3], *gamma_x = model[SEIDART_GX3],
                 *gamma_y = model[SEIDART_GY3], *gamma_z = model[SEIDART_GZ3],
                 *gamma_xy = model[SEIDART_GXY3], *gamma_yz = model[SEIDART_GYZ3],
                 *gamma_xz = model[SEIDART_GXZ3], *kappa = model[SEIDART_KAPPA3],
                 *kappa_half = model[SEIDART_KAPPAH3], *acoef = model[SEIDART_ACOEF3],
                 *acoef_half = model[SEIDART_ACOEFH3], *bcoef = model[SEIDART_BCOEF3],
                 *bcoef_half = model[SEIDART_BCOEFH3];
    double *vx = fields[S3_VX], *vy = fields[S3_VY], *vz = fields[S3_VZ],
           *sxx = fields[S3_SXX], *sxy = fields[S3_SXY], *sxz = fields[S3_SXZ],
           *syy = fields[S3_SYY], *syz = fields[S3_SYZ], *szz = fields[S3_SZZ];
    const int isource = s->xind + d->cpml, jsource = s->yind + d->cpml, ksource = s->zind + d->cpml;
    const size_t N = (size_t)nx * ny * nz;
    const double h24x = 24.0 * dx, h24y = 24.0 * dy, h24z = 24.0 * dz;

    for (int step = 0; step < nsteps; ++step) {
        const int it = it0 + step + 1;
        /* four stress loops, cpmlfdtd.f08:1761-1992.  Per loop: x/y/z stencil
         * direction (1 = forward "half grid") and CPML coefficient choice. */
        for (int L = 1; L <= 4; ++L) {
            int klo, khi, jlo, jhi, ilo, ihi, xf, yf, zf, xh, yh, zh;
            if (L == 1) { klo = 3; khi = nz - 1; jlo = 3; jhi = ny - 1; ilo = 2; ihi = nx - 2; xf = 1; yf = 0; zf = 0; xh = 1; yh = 0; zh = 0; }
            else if (L == 2) { klo = 3; khi = nz - 1; jlo = 2; jhi = ny - 2; ilo = 3; ihi = nx - 1; xf = 0; yf = 1; zf = 0; xh = 0; yh = 1; zh = 1; }
            else if (L == 3) { klo = 2; khi = nz - 2; jlo = 3; jhi = ny - 1; ilo = 3; ihi = nx - 1; xf = 0; yf = 0; zf = 1; xh = 0; yh = 0; zh = 1; }
            else { klo = 2; khi = nz - 2; jlo = 2; jhi = ny - 2; ilo = 2; ihi = nx - 2; xf = 1; yf = 1; zf = 1; xh = 1; yh = 1; zh = 1; }
            double* const* M = mem + 9 * (L - 1);
#pragma omp parallel for collapse(3) schedule(static)
            for (int k = klo; k <= khi; ++k)
                for (int j = jlo; j <= jhi; ++j)
                    for (int i = ilo; i <= ihi; ++i) {
                        const size_t c = IX3(i, j, k);
                        const double* v[3] = {vx, vy, vz};
                        double g[3][3]; /* g[comp][dir] */
                        for (int q = 0; q < 3; ++q) {
                            g[q][0] = xf ? d4(v[q], IX3(i + 1, j, k), c, IX3(i + 2, j, k), IX3(i - 1, j, k), h24x)
                                         : d4(v[q], c, IX3(i - 1, j, k), IX3(i + 1, j, k), IX3(i - 2, j, k), h24x);
                            g[q][1] = yf ? d4(v[q], IX3(i, j + 1, k), c, IX3(i, j + 2, k), IX3(i, j - 1, k), h24y)
                                         : d4(v[q], c, IX3(i, j - 1, k), IX3(i, j + 1, k), IX3(i, j - 2, k), h24y);
                            g[q][2] = zf ? d4(v[q], IX3(i, j, k + 1), c, IX3(i, j, k + 2), IX3(i, j, k - 1), h24z)
                                         : d4(v[q], c, IX3(i, j, k - 1), IX3(i, j, k + 1), IX3(i, j, k - 2), h24z);
                        }
                        const double bxv = xh ? bcoef_half[c] : bcoef[c], axv = xh ? acoef_half[c] : acoef[c], kxv = xh ? kappa_half[c] : kappa[c];
                        const double byv = yh ? bcoef_half[c] : bcoef[c], ayv = yh ? acoef_half[c] : acoef[c], kyv = yh ? kappa_half[c] : kappa[c];
                        const double bzv = zh ? bcoef_half[c] : bcoef[c], azv = zh ? acoef_half[c] : acoef[c], kzv = zh ? kappa_half[c] : kappa[c];
                        for (int q = 0; q < 3; ++q) {
                            g[q][0] = rcpml(M[3 * q + 0], c, bxv, axv, kxv, g[q][0]);
                            g[q][1] = rcpml(M[3 * q + 1], c, byv, ayv, kyv, g[q][1]);
                            if (L == 2 && q == 0) {
                                /* reference quirk (cpmlfdtd.f08:1855-1866): loop 2 updates
                                 * memory_dvx_dz2 but never rescales dvx_dz, so sigmaxy
                                 * uses the raw derivative */
                                M[2][c] = bzv * M[2][c] + azv * g[0][2];
                            } else {
                                g[q][2] = rcpml(M[3 * q + 2], c, bzv, azv, kzv, g[q][2]);
                            }
                        }
                        const double dvx_dx = g[0][0], dvx_dy = g[0][1], dvx_dz = g[0][2];
                        const double dvy_dx = g[1][0], dvy_dy = g[1][1], dvy_dz = g[1][2];
                        const double dvz_dx = g[2][0], dvz_dy = g[2][1], dvz_dz = g[2][2];
#define STRESS3(arr, a1, a2, a3, a4, a5, a6, gm)                                                        \
    arr[c] = (arr[c] + (CC(a1) * dvx_dx + CC(a2) * dvy_dy + CC(a3) * dvz_dz + CC(a4) * (dvy_dz + dvz_dy) + \
                        CC(a5) * (dvx_dz + dvz_dx) + CC(a6) * (dvy_dx + dvx_dy)) * dt) /                   \
             (1.0 + (gm)[c] * dt)
                        if (L == 1) {
                            STRESS3(sxx, C11, C12, C13, C14, C15, C16, gamma_x);
                            STRESS3(syy, C12, C22, C23, C24, C25, C26, gamma_y);
                            STRESS3(szz, C13, C23, C33, C34, C35, C36, gamma_z);
                        } else if (L == 2) {
                            STRESS3(sxy, C16, C26, C36, C46, C56, C66, gamma_xy);
                        } else if (L == 3) {
                            STRESS3(sxz, C15, C25, C35, C45, C55, C56, gamma_xz);
                        } else {
                            STRESS3(syz, C14, C24, C34, C44, C45, C46, gamma_yz);
                        }
#undef STRESS3
                    }
        }
        /* vx: cpmlfdtd.f08:2014-2034 */
#pragma omp parallel for collapse(3) schedule(static)
        for (int k = 3; k <= nz - 1; ++k)
            for (int j = 3; j <= ny - 1; ++j)
                for (int i = 3; i <= nx - 1; ++i) {
                    const size_t c = IX3(i, j, k);
                    const double rhoxx = scalar_mean(rho[c], rho[IX3(i - 1, j, k)], density_code);
                    const double rhoyx = scalar_mean(rho[c], rho[c], density_code);
                    const double rhozx = scalar_mean(rho[c], rho[IX3(i, j, k - 1)], density_code);
                    double a = (27.0 * sxx[c] - 27.0 * sxx[IX3(i - 1, j, k)] + sxx[IX3(i - 2, j, k)]) / h24x;
                    double b = (27.0 * sxy[c] - 27.0 * sxy[IX3(i, j - 1, k)] + sxy[IX3(i, j - 2, k)]) / h24y;
                    double e = (27.0 * sxz[c] - 27.0 * sxz[IX3(i, j, k - 1)] + sxz[IX3(i, j, k - 2)]) / h24z;
                    a = rcpml(mem[S3_M_DSXX_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], a);
                    b = rcpml(mem[S3_M_DSXY_DY], c, bcoef_half[c], acoef_half[c], kappa_half[c], b);
                    e = rcpml(mem[S3_M_DSXZ_DZ], c, bcoef_half[c], acoef_half[c], kappa_half[c], e);
                    vx[c] = vx[c] + (a / rhoxx + b / rhoyx + e / rhozx) * dt;
                }
        /* vy: cpmlfdtd.f08:2055-2076 */
#pragma omp parallel for collapse(3) schedule(static)
        for (int k = 3; k <= nz - 1; ++k)
            for (int j = 2; j <= ny - 2; ++j)
                for (int i = 2; i <= nx - 2; ++i) {
                    const size_t c = IX3(i, j, k);
                    const double rhoxy = scalar_mean(rho[c], rho[IX3(i + 1, j, k)], density_code);
                    const double rhoyy = scalar_mean(rho[c], rho[c], density_code);
                    const double rhozy = scalar_mean(rho[c], rho[IX3(i, j, k - 1)], density_code);
                    double a = (-27.0 * sxy[c] + 27.0 * sxy[IX3(i + 1, j, k)] - sxy[IX3(i + 2, j, k)]) / h24x;
                    double b = (-27.0 * syy[c] + 27.0 * syy[IX3(i, j + 1, k)] - syy[IX3(i, j + 2, k)]) / h24y;
                    double e = (27.0 * syz[c] - 27.0 * syz[IX3(i, j, k - 1)] + syz[IX3(i, j, k - 2)]) / h24z;
                    a = rcpml(mem[S3_M_DSXY_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], a);
                    b = rcpml(mem[S3_M_DSYY_DY], c, bcoef_half[c], acoef_half[c], kappa_half[c], b);
                    e = rcpml(mem[S3_M_DSYZ_DZ], c, bcoef[c], acoef[c], kappa[c], e);
                    vy[c] = vy[c] + (a / rhoxy + b / rhoyy + e / rhozy) * dt;
                }
        /* vz: cpmlfdtd.f08:2098-2120 */
#pragma omp parallel for collapse(3) schedule(static)
        for (int k = 2; k <= nz - 2; ++k)
            for (int j = 3; j <= ny - 1; ++j)
                for (int i = 2; i <= nx - 2; ++i) {
                    const size_t c = IX3(i, j, k);
                    const double rhoxz = scalar_mean(rho[c], rho[IX3(i + 1, j, k)], density_code);
                    const double rhoyz = scalar_mean(rho[c], rho[c], density_code);
                    const double rhozz = scalar_mean(rho[c], rho[IX3(i, j, k + 1)], density_code);
                    double a = (-27.0 * sxz[c] + 27.0 * sxz[IX3(i + 1, j, k)] - sxz[IX3(i + 2, j, k)]) / h24x;
                    double b = (27.0 * syz[c] - 27.0 * syz[IX3(i, j - 1, k)] + syz[IX3(i, j - 2, k)]) / h24y;
                    double e = (-27.0 * szz[c] + 27.0 * szz[IX3(i, j, k + 1)] - szz[IX3(i, j, k + 2)]) / h24z;
                    a = rcpml(mem[S3_M_DSXZ_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], a);
                    b = rcpml(mem[S3_M_DSYZ_DY], c, bcoef[c], acoef[c], kappa[c], b);
                    e = rcpml(mem[S3_M_DSZZ_DZ], c, bcoef_half[c], acoef_half[c], kappa_half[c], e);
                    vz[c] = vz[c] + (a / rhoxz + b / rhoyz + e / rhozz) * dt;
                }
        if (g_pw_on) {  /* plane wave: cpmlfdtd.f08:2133-2203 */
            PwGeom G;
            pw_geom(d, 1, 2, &G);
            const double t = it * dt;
            double V[3], st[6];
            PW_FACES3(G, dx, dy, dz, {
                pw_seismic_field(r, G.r0, t, V, st);
                vx[c] = vx[c] + V[0];
                vy[c] = vy[c] + V[1];
                vz[c] = vz[c] + V[2];
                double sg[6] = {sxx[c], syy[c], szz[c], syz[c], sxz[c], sxy[c]};
                pw_add_stress(C, c, st, sg);
                sxx[c] = sg[0]; syy[c] = sg[1]; szz[c] = sg[2]; syz[c] = sg[3]; sxz[c] = sg[4]; sxy[c] = sg[5];
            });
        } else
        /* point source: cpmlfdtd.f08:2210-2219 */
        {
            const int is = isource, js = jsource, ks = ksource;
            sxx[IX3(is, js, ks)] += src_at(srcfn[S3_SRCXX], it) / rho[IX3(is, js, ks)];
            sxy[IX3(is + 1, js + 1, ks)] += src_at(srcfn[S3_SRCXY], it) / rho[IX3(is + 1, js + 1, ks)];
            sxz[IX3(is + 1, js, ks + 1)] += src_at(srcfn[S3_SRCXZ], it) / rho[IX3(is + 1, js, ks)];
            syy[IX3(is, js, ks)] += src_at(srcfn[S3_SRCYY], it) / rho[IX3(is, js, ks)];
            syz[IX3(is, js + 1, ks + 1)] += src_at(srcfn[S3_SRCYZ], it) / rho[IX3(is, js, ks + 1)];
            szz[IX3(is, js, ks)] += src_at(srcfn[S3_SRCZZ], it) / rho[IX3(is, js, ks)];
            vx[IX3(is + 1, js, ks)] += src_at(srcfn[S3_SRCX], it) * dt / rho[IX3(is + 1, js, ks)];
            vy[IX3(is, js + 1, ks)] += src_at(srcfn[S3_SRCY], it) * dt / rho[IX3(is, js, ks)];
            vz[IX3(is, js, ks + 1)] += src_at(srcfn[S3_SRCZ], it) * dt / rho[IX3(is, js, ks + 1)];
        }
        /* Dirichlet on the six faces: cpmlfdtd.f08:2226-2248 */
        {
            double* vv[3] = {vx, vy, vz};
            for (int q = 0; q < 3; ++q) {
                for (int k = 1; k <= nz; ++k)
                    for (int j = 1; j <= ny; ++j) { vv[q][IX3(1, j, k)] = 0.0; vv[q][IX3(nx, j, k)] = 0.0; }
                for (int k = 1; k <= nz; ++k)
                    for (int i = 1; i <= nx; ++i) { vv[q][IX3(i, 1, k)] = 0.0; vv[q][IX3(i, ny, k)] = 0.0; }
                for (int j = 1; j <= ny; ++j)
                    for (int i = 1; i <= nx; ++i) { vv[q][IX3(i, j, 1)] = 0.0; vv[q][IX3(i, j, nz)] = 0.0; }
            }
        }
        /* norms: cpmlfdtd.f08:2255-2258 */
        double vn = 0.0, sn = 0.0;
#pragma omp parallel for reduction(max : vn, sn) schedule(static)
        for (size_t c = 0; c < N; ++c) {
            const double a = sqrt(vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c]);
            const double b = sqrt(sxx[c] * sxx[c] + syy[c] * syy[c] + szz[c] * szz[c] +
                                  2.0 * (sxy[c] * sxy[c] + syz[c] * syz[c] + sxz[c] * sxz[c]));
            vn = vn > a ? vn : a;
            sn = sn > b ? sn : b;
        }
        if (norms) { norms[step] = vn; norms[nsteps + step] = sn; }
        if (traces)
            for (int r = 0; r < nrec; ++r) {
                traces[((size_t)step * 3 + 0) * nrec + r] = vx[rec[r]];
                traces[((size_t)step * 3 + 1) * nrec + r] = vy[rec[r]];
                traces[((size_t)step * 3 + 2) * nrec + r] = vz[rec[r]];
            }
        if (vn > STABILITY_THRESHOLD) return it;
    }
#undef CC
    return 0;
}

/* =====================================================================
 * electromag2: cpmlfdtd.f08:2519-2748
 * ===================================================================== */
int oracle_electromag2(const SeidartDomain* d, const SeidartSource* s,
                       const double* const* model, const double* const* srcfn,
                       double* const* fields, double* const* mem, int it0, int nsteps,
                       int nrec, const int* rec, double* traces, double* norms) {
    const int nx = d->nx, nz = d->nz;
    const double dx = d->dx, dz = d->dz, dt = s->dt;
    const double *eps11 = model[E2_E11], *eps13 = model[E2_E13], *eps33 = model[E2_E33],
                 *sig11 = model[E2_S11], *sig13 = model[E2_S13], *sig33 = model[E2_S33],
                 *kappa = model[E2_KAPPA], *kappa_half = model[E2_KAPPAH],
                 *acoef = model[E2_ACOEF], *acoef_half = model[E2_ACOEFH],
                 *bcoef = model[E2_BCOEF], *bcoef_half = model[E2_BCOEFH];
    double *Ex = fields[E2_EX], *Ez = fields[E2_EZ], *Hy = fields[E2_HY];
    double *m_dEx_dz = mem[E2_M_DEX_DZ], *m_dEz_dx = mem[E2_M_DEZ_DX],
           *m_dHy_dx = mem[E2_M_DHY_DX], *m_dHy_dz = mem[E2_M_DHY_DZ];
    const int isource = s->xind + d->cpml, jsource = s->zind + d->cpml;
    const size_t N = (size_t)nx * nz;

    /* coefficient set-up: cpmlfdtd.f08:2519-2540 */
    const double dbHy = dt / MU0, daHy = 1.0;
    double* buf = (double*)malloc(sizeof(double) * N * 12);
    if (!buf) return -1;
    double *e11 = buf, *e33 = buf + N, *aEx = buf + 2 * N, *bEx = buf + 3 * N, *dEx = buf + 4 * N,
           *eEx = buf + 5 * N, *aEz = buf + 6 * N, *bEz = buf + 7 * N, *dEz = buf + 8 * N,
           *eEz = buf + 9 * N, *Exo = buf + 10 * N, *Ezo = buf + 11 * N;
    for (size_t c = 0; c < N; ++c) {
        const double a11 = eps11[c] * EPS0, a13 = eps13[c] * EPS0, a33 = eps33[c] * EPS0;
        double det = a11 * a33 - a13 * a13;
        if (det <= 1.0e-18 * EPS0 * EPS0) det = 1.0e-18 * EPS0 * EPS0;
        e11[c] = a11; e33[c] = a33;
        aEx[c] = a33 / det;
        bEx[c] = -a13 / det;
        dEx[c] = (a33 * sig11[c] - a13 * sig13[c]) / det;
        eEx[c] = (a33 * sig13[c] - a13 * sig33[c]) / det;
        aEz[c] = -a13 / det;
        bEz[c] = a11 / det;
        dEz[c] = (a11 * sig13[c] - a13 * sig11[c]) / det;
        eEz[c] = (a11 * sig33[c] - a13 * sig13[c]) / det;
    }
    memcpy(Exo, Ex, sizeof(double) * N);
    memcpy(Ezo, Ez, sizeof(double) * N);

    int status = 0;
    for (int step = 0; step < nsteps; ++step) {
        const int it = it0 + step + 1;
        /* H update: cpmlfdtd.f08:2576-2593 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int j = 1; j <= nz - 1; ++j)
            for (int i = 1; i <= nx - 1; ++i) {
                const size_t c = IX2(i, j);
                double dEx_dz = (Ex[IX2(i, j + 1)] - Ex[c]) / dz;
                double dEz_dx = (Ez[IX2(i + 1, j)] - Ez[c]) / dx;
                m_dEx_dz[c] = bcoef[c] * m_dEx_dz[c] + acoef[c] * dEx_dz;
                m_dEz_dx[c] = bcoef_half[c] * m_dEz_dx[c] + acoef_half[c] * dEz_dx;
                dEz_dx = dEz_dx / kappa_half[c] + m_dEz_dx[c];
                dEx_dz = dEx_dz / kappa[c] + m_dEx_dz[c];
                Hy[c] = daHy * Hy[c] + dbHy * (dEz_dx - dEx_dz);
            }
        /* E update: cpmlfdtd.f08:2605-2620 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int j = 2; j <= nz; ++j)
            for (int i = 2; i <= nx; ++i) {
                const size_t c = IX2(i, j);
                double dHy_dz = (Hy[c] - Hy[IX2(i, j - 1)]) / dz;
                double dHy_dx = (Hy[c] - Hy[IX2(i - 1, j)]) / dx;
                m_dHy_dx[c] = bcoef_half[c] * m_dHy_dx[c] + acoef_half[c] * dHy_dx;
                m_dHy_dz[c] = bcoef[c] * m_dHy_dz[c] + acoef[c] * dHy_dz;
                dHy_dz = dHy_dz / kappa[c] + m_dHy_dz[c];
                dHy_dx = dHy_dx / kappa_half[c] + m_dHy_dx[c];
                Ez[c] = Ezo[c] + (-aEz[c] * dHy_dz + bEz[c] * dHy_dx - dEz[c] * Exo[c] - eEz[c] * Ezo[c]) * dt;
                Ex[c] = Exo[c] + (-aEx[c] * dHy_dz + bEx[c] * dHy_dx - dEx[c] * Exo[c] - eEx[c] * Ezo[c]) * dt;
            }
        if (g_pw_on) {  /* plane wave: cpmlfdtd.f08:2626-2673 */
            PwGeom G;
            pw_geom(d, 0, 2, &G);
            const double t = it * s->dt;
            double r[3], E[3], H[3];
            for (int face = 0; face < 2; ++face) {
                const int xface = face == 0;
                if (xface ? !(G.active[0] || G.active[1]) : !(G.active[4] || G.active[5])) continue;
                const int fixed = xface ? nint_(G.loc[0] / dx) : nint_(G.loc[2] / dz);
                const int lo = xface ? G.kmin : G.imin, hi = xface ? G.kmax : G.imax;
                for (int ip = lo; ip <= hi; ++ip) {
                    if (xface) { r[0] = G.loc[0]; r[1] = 0.0; r[2] = ip * dz; }
                    else { r[0] = ip * dx; r[1] = 0.0; r[2] = G.loc[2]; }
                    pw_em_field(r, G.r0, t, E, H);
                    const size_t c = xface ? IX2(fixed, ip) : IX2(ip, fixed);
                    Ex[c] = Ex[c] + E[0];
                    Ez[c] = Ez[c] + E[2];
                    Hy[c] = Hy[c] + H[1];
                }
            }
        } else
        /* point source: cpmlfdtd.f08:2678-2681 */
        {
            const size_t c = IX2(isource, jsource);
            Ex[c] = Ex[c] + src_at(srcfn[E2_SRCX], it) * dt / e11[c];
            Ez[c] = Ez[c] + src_at(srcfn[E2_SRCZ], it) * dt / e33[c];
        }
        /* Dirichlet: cpmlfdtd.f08:2690-2707 */
        for (int j = 1; j <= nz; ++j) {
            Ex[IX2(1, j)] = 0.0; Ex[IX2(nx, j)] = 0.0;
            Ez[IX2(1, j)] = 0.0; Ez[IX2(nx, j)] = 0.0;
            Hy[IX2(1, j)] = 0.0; Hy[IX2(nx, j)] = 0.0;
        }
        for (int i = 1; i <= nx; ++i) {
            Ex[IX2(i, 1)] = 0.0; Ex[IX2(i, nz)] = 0.0;
            Ez[IX2(i, 1)] = 0.0; Ez[IX2(i, nz)] = 0.0;
            Hy[IX2(i, 1)] = 0.0; Hy[IX2(i, nz)] = 0.0;
        }
        /* E_old = E: cpmlfdtd.f08:2711-2716 */
        memcpy(Exo, Ex, sizeof(double) * N);
        memcpy(Ezo, Ez, sizeof(double) * N);
        /* norm: cpmlfdtd.f08:2726-2740 */
        double velocnorm = 0.0;
#pragma omp parallel for reduction(max : velocnorm) schedule(static)
        for (size_t c = 0; c < N; ++c) {
            const double n = sqrt(Ex[c] * Ex[c] + Ez[c] * Ez[c]);
            velocnorm = velocnorm > n ? velocnorm : n;
        }
        if (norms) norms[step] = velocnorm;
        if (traces)
            for (int r = 0; r < nrec; ++r) {
                traces[((size_t)step * 2 + 0) * nrec + r] = Ex[rec[r]];
                traces[((size_t)step * 2 + 1) * nrec + r] = Ez[rec[r]];
            }
        if (velocnorm > STABILITY_THRESHOLD) { status = it; break; }
    }
    free(buf);
    return status;
}

/* =====================================================================
 * electromag25: cpmlfdtd.f08:3046-3331 (complex fields, d/dy = i ky)
 * ===================================================================== */
int oracle_electromag25(const SeidartDomain* d, const SeidartSource* s,
                        const double* const* model, const double* const* srcfn,
                        double* const* fields, double* const* mem, int it0, int nsteps,
                        int nrec, const int* rec, double* traces, double* norms) {
    const int nx = d->nx, nz = d->nz;
    const double dx = d->dx, dz = d->dz, dt = s->dt, ky = s->ky;
    const double *sig11 = model[E25_S11], *sig12 = model[E25_S12], *sig13 = model[E25_S13],
                 *sig22 = model[E25_S22], *sig23 = model[E25_S23], *sig33 = model[E25_S33],
                 *kappa = model[E25_KAPPA], *kappa_half = model[E25_KAPPAH],
                 *acoef = model[E25_ACOEF], *acoef_half = model[E25_ACOEFH],
                 *bcoef = model[E25_BCOEF], *bcoef_half = model[E25_BCOEFH];
    double *Ex = fields[E25_EX], *Ey = fields[E25_EY], *Ez = fields[E25_EZ],
           *Hx = fields[E25_HX], *Hy = fields[E25_HY], *Hz = fields[E25_HZ];
    const int isource = s->xind + d->cpml, ksource = s->zind + d->cpml;
    const size_t N = (size_t)nx * nz;

    /* coefficient set-up: cpmlfdtd.f08:3046-3067 */
    double* buf = (double*)malloc(sizeof(double) * N * (12 + 6));
    if (!buf) return -1;
    double *e11 = buf, *e22 = buf + N, *e33 = buf + 2 * N;
    double *aEx = buf + 3 * N, *bEx = buf + 4 * N, *cEx = buf + 5 * N, *bEy = buf + 6 * N,
           *cEy = buf + 7 * N, *cEz = buf + 8 * N;
    double* Eo = buf + 12 * N; /* 3 complex arrays: Ex_old, Ey_old, Ez_old */
    for (size_t c = 0; c < N; ++c) {
        const double a11 = model[E25_E11][c] * EPS0, a12 = model[E25_E12][c] * EPS0,
                     a13 = model[E25_E13][c] * EPS0, a22 = model[E25_E22][c] * EPS0,
                     a23 = model[E25_E23][c] * EPS0, a33 = model[E25_E33][c] * EPS0;
        const double det = a11 * (a22 * a33 - a23 * a23) - a12 * (a12 * a33 - a23 * a13) +
                           a13 * (a12 * a23 - a22 * a13);
        e11[c] = a11; e22[c] = a22; e33[c] = a33;
        aEx[c] = (a22 * a33 - a23 * a23) / det;
        bEx[c] = -((a12 * a33 - a23 * a13) / det);
        cEx[c] = (a12 * a23 - a22 * a13) / det;
        bEy[c] = (a11 * a33 - a13 * a13) / det;
        cEy[c] = -((a11 * a23 - a12 * a13) / det);
        cEz[c] = (a11 * a22 - a12 * a12) / det;
    }
    const double *aEy = bEx, *aEz = cEx, *bEz = cEy;
    double *Exo = Eo, *Eyo = Eo + 2 * N, *Ezo = Eo + 4 * N;
    memcpy(Exo, Ex, sizeof(double) * 2 * N);
    memcpy(Eyo, Ey, sizeof(double) * 2 * N);
    memcpy(Ezo, Ez, sizeof(double) * 2 * N);
    const double h24x = 24.0 * dx, h24z = 24.0 * dz;

    int status = 0;
    for (int step = 0; step < nsteps; ++step) {
        const int it = it0 + step + 1;
        /* Hx: cpmlfdtd.f08:3106-3119 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 2; k <= nz - 2; ++k)
            for (int i = 2; i <= nx - 1; ++i) {
                const size_t c = IX2(i, k);
                cplx dEy_dz = cd4(Ey, IX2(i, k + 1), c, IX2(i, k + 2), IX2(i, k - 1), h24z);
                dEy_dz = ccpml(mem[E25_M_DEY_DZ], c, bcoef_half[c], acoef_half[c], kappa_half[c], dEy_dz);
                cst(Hx, c, csub(cld(Hx, c), crmul(dt / MU0, csub(ciky(ky, cld(Ez, c)), dEy_dz))));
            }
        /* Hy: cpmlfdtd.f08:3132-3151 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 2; k <= nz - 2; ++k)
            for (int i = 2; i <= nx - 2; ++i) {
                const size_t c = IX2(i, k);
                cplx dEx_dz = cd4(Ex, IX2(i, k + 1), c, IX2(i, k + 2), IX2(i, k - 1), h24z);
                cplx dEz_dx = cd4(Ez, IX2(i + 1, k), c, IX2(i + 2, k), IX2(i - 1, k), h24x);
                dEx_dz = ccpml(mem[E25_M_DEX_DZ], c, bcoef_half[c], acoef_half[c], kappa_half[c], dEx_dz);
                dEz_dx = ccpml(mem[E25_M_DEZ_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], dEz_dx);
                cst(Hy, c, csub(cld(Hy, c), crmul(dt / MU0, csub(dEx_dz, dEz_dx))));
            }
        /* Hz: cpmlfdtd.f08:3164-3177 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
            for (int i = 2; i <= nx - 2; ++i) {
                const size_t c = IX2(i, k);
                cplx dEy_dx = cd4(Ey, IX2(i + 1, k), c, IX2(i + 2, k), IX2(i - 1, k), h24x);
                dEy_dx = ccpml(mem[E25_M_DEY_DX], c, bcoef_half[c], acoef_half[c], kappa_half[c], dEy_dx);
                cst(Hz, c, csub(cld(Hz, c), crmul(dt / MU0, csub(dEy_dx, ciky(ky, cld(Ex, c))))));
            }
        /* E: cpmlfdtd.f08:3195-3245 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 3; k <= nz - 2; ++k)
            for (int i = 3; i <= nx - 2; ++i) {
                const size_t c = IX2(i, k);
                const cplx dHz_dy = ciky(ky, cld(Hz, c));
                cplx dHy_dz = cd4(Hy, c, IX2(i, k - 1), IX2(i, k + 1), IX2(i, k - 2), h24z);
                cplx dHx_dz = cd4(Hx, c, IX2(i, k - 1), IX2(i, k + 1), IX2(i, k - 2), h24z);
                cplx dHz_dx = cd4(Hz, c, IX2(i - 1, k), IX2(i + 1, k), IX2(i - 2, k), h24x);
                cplx dHy_dx = cd4(Hy, c, IX2(i - 1, k), IX2(i + 1, k), IX2(i - 2, k), h24x);
                const cplx dHx_dy = ciky(ky, cld(Hx, c));
                dHy_dz = ccpml(mem[E25_M_DHY_DZ], c, bcoef[c], acoef[c], kappa[c], dHy_dz);
                dHx_dz = ccpml(mem[E25_M_DHX_DZ], c, bcoef[c], acoef[c], kappa[c], dHx_dz);
                dHz_dx = ccpml(mem[E25_M_DHZ_DX], c, bcoef[c], acoef[c], kappa[c], dHz_dx);
                dHy_dx = ccpml(mem[E25_M_DHY_DX], c, bcoef[c], acoef[c], kappa[c], dHy_dx);
                const cplx exo = cld(Exo, c), eyo = cld(Eyo, c), ezo = cld(Ezo, c);
                const cplx rhs_x = csub(csub(dHz_dy, dHy_dz),
                                        cadd(cadd(crmul(sig11[c], exo), crmul(sig12[c], eyo)), crmul(sig13[c], ezo)));
                const cplx rhs_y = csub(csub(dHx_dz, dHz_dx),
                                        cadd(cadd(crmul(sig12[c], exo), crmul(sig22[c], eyo)), crmul(sig23[c], ezo)));
                const cplx rhs_z = csub(csub(dHy_dx, dHx_dy),
                                        cadd(cadd(crmul(sig13[c], exo), crmul(sig23[c], eyo)), crmul(sig33[c], ezo)));
                cst(Ex, c, cadd(exo, cmulr(cadd(cadd(crmul(aEx[c], rhs_x), crmul(bEx[c], rhs_y)), crmul(cEx[c], rhs_z)), dt)));
                cst(Ey, c, cadd(eyo, cmulr(cadd(cadd(crmul(aEy[c], rhs_x), crmul(bEy[c], rhs_y)), crmul(cEy[c], rhs_z)), dt)));
                cst(Ez, c, cadd(ezo, cmulr(cadd(cadd(crmul(aEz[c], rhs_x), crmul(bEz[c], rhs_y)), crmul(cEz[c], rhs_z)), dt)));
            }
        /* point source: cpmlfdtd.f08:3261-3266 (real part only) */
        {
            const size_t c = IX2(isource, ksource);
            Ex[2 * c] = Ex[2 * c] + src_at(srcfn[E25_SRCX], it) * dt / e11[c];
            Ey[2 * c] = Ey[2 * c] + src_at(srcfn[E25_SRCY], it) * dt / e22[c];
            Ez[2 * c] = Ez[2 * c] + src_at(srcfn[E25_SRCZ], it) * dt / e33[c];
        }
        /* Dirichlet on E and H: cpmlfdtd.f08:3270-3298 */
        {
            double* ff[6] = {Ex, Ey, Ez, Hx, Hy, Hz};
            for (int q = 0; q < 6; ++q) {
                for (int k = 1; k <= nz; ++k) {
                    ff[q][2 * IX2(1, k)] = ff[q][2 * IX2(1, k) + 1] = 0.0;
                    ff[q][2 * IX2(nx, k)] = ff[q][2 * IX2(nx, k) + 1] = 0.0;
                }
                for (int i = 1; i <= nx; ++i) {
                    ff[q][2 * IX2(i, 1)] = ff[q][2 * IX2(i, 1) + 1] = 0.0;
                    ff[q][2 * IX2(i, nz)] = ff[q][2 * IX2(i, nz) + 1] = 0.0;
                }
            }
        }
        memcpy(Exo, Ex, sizeof(double) * 2 * N);
        memcpy(Eyo, Ey, sizeof(double) * 2 * N);
        memcpy(Ezo, Ez, sizeof(double) * 2 * N);
        /* norm: cpmlfdtd.f08:3308-3309 */
        double velocnorm = 0.0;
#pragma omp parallel for reduction(max : velocnorm) schedule(static)
        for (size_t c = 0; c < N; ++c) {
            const double a = Ex[2 * c] * Ex[2 * c] + Ex[2 * c + 1] * Ex[2 * c + 1];
            const double b = Ey[2 * c] * Ey[2 * c] + Ey[2 * c + 1] * Ey[2 * c + 1];
            const double e = Ez[2 * c] * Ez[2 * c] + Ez[2 * c + 1] * Ez[2 * c + 1];
            const double n = sqrt(a + b + e);
            velocnorm = velocnorm > n ? velocnorm : n;
        }
        if (norms) norms[step] = velocnorm;
        if (traces)
            for (int r = 0; r < nrec; ++r) {
                const double* ff[3] = {Ex, Ey, Ez};
                for (int q = 0; q < 3; ++q) {
                    traces[2 * (((size_t)step * 3 + q) * nrec + r)] = ff[q][2 * (size_t)rec[r]];
                    traces[2 * (((size_t)step * 3 + q) * nrec + r) + 1] = ff[q][2 * (size_t)rec[r] + 1];
                }
            }
        if (velocnorm > STABILITY_THRESHOLD) { status = it; break; }
    }
    free(buf);
    return status;
}

/* =====================================================================
 * electromag3: cpmlfdtd.f08:3353-4001 (point sources; the plane-wave
 * branch is not restated)
 * ===================================================================== */
int oracle_electromag3(const SeidartDomain* d, const SeidartSource* s,
                       const double* const* model, const double* const* srcfn,
                       double* const* fields, double* const* mem, int it0, int nsteps,
                       int nrec, const int* rec, double* traces, double* norms) {
    const int nx = d->nx, ny = d->ny, nz = d->nz;
    const double dx = d->dx, dy = d->dy, dz = d->dz, dt = s->dt;
    const double *sig11 = model[E3_S11], *sig12 = model[E3_S12], *sig13 = model[E3_S13],
                 *sig22 = model[E3_S22], *sig23 = model[E3_S23], *sig33 = model[E3_S33],
                 *kappa = model[E3_KAPPA], *kappa_half = model[E3_KAPPAH],
                 *acoef = model[E3_ACOEF], *acoef_half = model[E3_ACOEFH],
                 *bcoef = model[E3_BCOEF], *bcoef_half = model[E3_BCOEFH];
    double *Ex = fields[E3_EX], *Ey = fields[E3_EY], *Ez = fields[E3_EZ],
           *Hx = fields[E3_HX], *Hy = fields[E3_HY], *Hz = fields[E3_HZ];
    double *m_dEx_dy = mem[E3_M_DEX_DY], *m_dEy_dx = mem[E3_M_DEY_DX], *m_dEx_dz = mem[E3_M_DEX_DZ],
           *m_dEz_dx = mem[E3_M_DEZ_DX], *m_dEz_dy = mem[E3_M_DEZ_DY], *m_dEy_dz = mem[E3_M_DEY_DZ],
           *m_dHz_dx = mem[E3_M_DHZ_DX], *m_dHx_dz = mem[E3_M_DHX_DZ], *m_dHz_dy = mem[E3_M_DHZ_DY],
           *m_dHy_dz = mem[E3_M_DHY_DZ], *m_dHx_dy = mem[E3_M_DHX_DY], *m_dHy_dx = mem[E3_M_DHY_DX];
    const int isource = s->xind + d->cpml, jsource = s->yind + d->cpml, ksource = s->zind + d->cpml;
    const size_t N = (size_t)nx * ny * nz;
    /* cpmlfdtd.f08:3484-3494, :3644-3666 */
    const double dbHx = dt / MU0, daHx = 1.0, dbHy = dt / MU0, daHy = 1.0, dbHz = dt / MU0, daHz = 1.0;
    double* buf = (double*)malloc(sizeof(double) * N * 15);
    if (!buf) return -1;
    double *e11 = buf, *e22 = buf + N, *e33 = buf + 2 * N;
    double *aEx = buf + 3 * N, *bEx = buf + 4 * N, *cEx = buf + 5 * N, *bEy = buf + 6 * N,
           *cEy = buf + 7 * N, *cEz = buf + 8 * N;
    double *Ex_old = buf + 9 * N, *Ey_old = buf + 10 * N, *Ez_old = buf + 11 * N;
    for (size_t c = 0; c < N; ++c) {
        const double a11 = model[E3_E11][c] * EPS0, a12 = model[E3_E12][c] * EPS0,
                     a13 = model[E3_E13][c] * EPS0, a22 = model[E3_E22][c] * EPS0,
                     a23 = model[E3_E23][c] * EPS0, a33 = model[E3_E33][c] * EPS0;
        const double det = a11 * (a22 * a33 - a23 * a23) - a12 * (a12 * a33 - a23 * a13) +
                           a13 * (a12 * a23 - a22 * a13);
        e11[c] = a11; e22[c] = a22; e33[c] = a33;
        aEx[c] = (a22 * a33 - a23 * a23) / det;
        bEx[c] = -((a12 * a33 - a23 * a13) / det);
        cEx[c] = (a12 * a23 - a22 * a13) / det;
        bEy[c] = (a11 * a33 - a13 * a13) / det;
        cEy[c] = -((a11 * a23 - a12 * a13) / det);
        cEz[c] = (a11 * a22 - a12 * a12) / det;
    }
    const double *aEy = bEx, *aEz = cEx, *bEz = cEy;
    /* Ex_old = Ex at the start of every step (cpmlfdtd.f08:3668-3670, :3980-3982) */
    memcpy(Ex_old, Ex, sizeof(double) * N);
    memcpy(Ey_old, Ey, sizeof(double) * N);
    memcpy(Ez_old, Ez, sizeof(double) * N);

    for (int step = 0; step < nsteps; ++step) {
        const int it = it0 + step + 1;
        /* Hx: cpmlfdtd.f08:3695-3711 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 1; k <= nz - 1; ++k)
            for (int i = 1; i <= nx - 1; ++i)
                for (int j = 1; j <= ny - 1; ++j) {
                    const size_t c = IX3(i, j, k);
                    double dEz_dy = (Ez[IX3(i, j + 1, k)] - Ez[c]) / dy;
                    double dEy_dz = (Ey[IX3(i, j, k + 1)] - Ey[c]) / dz;
                    m_dEy_dz[c] = bcoef_half[c] * m_dEy_dz[c] + acoef_half[c] * dEy_dz;
                    m_dEz_dy[c] = bcoef_half[c] * m_dEz_dy[c] + acoef_half[c] * dEz_dy;
                    dEz_dy = dEz_dy / kappa_half[c] + m_dEz_dy[c];
                    dEy_dz = dEy_dz / kappa_half[c] + m_dEy_dz[c];
                    Hx[c] = daHx * Hx[c] + dbHx * (dEy_dz - dEz_dy);
                }
        /* Hy: cpmlfdtd.f08:3722-3741 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 1; k <= nz - 1; ++k)
            for (int i = 1; i <= nx - 1; ++i)
                for (int j = 1; j <= ny - 1; ++j) {
                    const size_t c = IX3(i, j, k);
                    double dEx_dz = (Ex[IX3(i, j, k + 1)] - Ex[c]) / dz;
                    double dEz_dx = (Ez[IX3(i + 1, j, k)] - Ez[c]) / dx;
                    m_dEx_dz[c] = bcoef[c] * m_dEx_dz[c] + acoef[c] * dEx_dz;
                    m_dEz_dx[c] = bcoef[c] * m_dEz_dx[c] + acoef[c] * dEz_dx;
                    dEx_dz = dEx_dz / kappa[c] + m_dEx_dz[c];
                    dEz_dx = dEz_dx / kappa[c] + m_dEz_dx[c];
                    Hy[c] = daHy * Hy[c] + dbHy * (dEz_dx - dEx_dz);
                }
        /* Hz: cpmlfdtd.f08:3752-3769 (k starts at 2) */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
            for (int i = 1; i <= nx - 1; ++i)
                for (int j = 1; j <= ny - 1; ++j) {
                    const size_t c = IX3(i, j, k);
                    double dEx_dy = (Ex[IX3(i, j + 1, k)] - Ex[c]) / dy;
                    double dEy_dx = (Ey[IX3(i + 1, j, k)] - Ey[c]) / dx;
                    m_dEx_dy[c] = bcoef[c] * m_dEx_dy[c] + acoef[c] * dEx_dy;
                    m_dEy_dx[c] = bcoef[c] * m_dEy_dx[c] + acoef[c] * dEy_dx;
                    dEx_dy = dEx_dy / kappa[c] + m_dEx_dy[c];
                    dEy_dx = dEy_dx / kappa[c] + m_dEy_dx[c];
                    Hz[c] = daHz * Hz[c] + dbHz * (dEx_dy - dEy_dx);
                }
        /* E: cpmlfdtd.f08:3787-3825 */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 2; k <= nz - 1; ++k)
            for (int i = 2; i <= nx - 1; ++i)
                for (int j = 2; j <= ny - 1; ++j) {
                    const size_t c = IX3(i, j, k);
                    double dHz_dy = (Hz[c] - Hz[IX3(i, j - 1, k)]) / dy;
                    double dHy_dz = (Hy[c] - Hy[IX3(i, j, k - 1)]) / dz;
                    double dHz_dx = (Hz[c] - Hz[IX3(i - 1, j, k)]) / dx;
                    double dHx_dz = (Hx[c] - Hx[IX3(i, j, k - 1)]) / dz;
                    double dHy_dx = (Hy[c] - Hy[IX3(i - 1, j, k)]) / dx;
                    double dHx_dy = (Hx[c] - Hx[IX3(i, j - 1, k)]) / dy;
                    m_dHz_dy[c] = bcoef_half[c] * m_dHz_dy[c] + acoef_half[c] * dHz_dy;
                    m_dHy_dz[c] = bcoef[c] * m_dHy_dz[c] + acoef[c] * dHy_dz;
                    m_dHz_dx[c] = bcoef_half[c] * m_dHz_dx[c] + acoef_half[c] * dHz_dx;
                    m_dHx_dz[c] = bcoef_half[c] * m_dHx_dz[c] + acoef_half[c] * dHx_dz;
                    m_dHx_dy[c] = bcoef_half[c] * m_dHx_dy[c] + acoef_half[c] * dHx_dy;
                    m_dHy_dx[c] = bcoef_half[c] * m_dHy_dx[c] + acoef_half[c] * dHy_dx;
                    dHz_dy = dHz_dy / kappa_half[c] + m_dHz_dy[c];
                    dHy_dz = dHy_dz / kappa[c] + m_dHy_dz[c];
                    dHz_dx = dHz_dx / kappa_half[c] + m_dHz_dx[c];
                    dHx_dz = dHx_dz / kappa_half[c] + m_dHx_dz[c];
                    dHx_dy = dHx_dy / kappa_half[c] + m_dHx_dy[c];
                    dHy_dx = dHy_dx / kappa_half[c] + m_dHy_dx[c];
                    const double rhs_x = dHz_dy - dHy_dz - (sig11[c] * Ex_old[c] + sig12[c] * Ey_old[c] + sig13[c] * Ez_old[c]);
                    const double rhs_y = dHx_dz - dHz_dx - (sig12[c] * Ex_old[c] + sig22[c] * Ey_old[c] + sig23[c] * Ez_old[c]);
                    const double rhs_z = dHy_dx - dHx_dy - (sig13[c] * Ex_old[c] + sig23[c] * Ey_old[c] + sig33[c] * Ez_old[c]);
                    Ex[c] = Ex_old[c] + (aEx[c] * rhs_x + bEx[c] * rhs_y + cEx[c] * rhs_z) * dt;
                    Ey[c] = Ey_old[c] + (aEy[c] * rhs_x + bEy[c] * rhs_y + cEy[c] * rhs_z) * dt;
                    Ez[c] = Ez_old[c] + (aEz[c] * rhs_x + bEz[c] * rhs_y + cEz[c] * rhs_z) * dt;
                }
        if (g_pw_on) {  /* plane wave: cpmlfdtd.f08:3833-3900 */
            PwGeom G;
            pw_geom(d, 1, 3, &G);
            const double t = it * s->dt;
            double E[3], H[3];
            PW_FACES3(G, dx, dy, dz, {
                pw_em_field(r, G.r0, t, E, H);
                Ex[c] = Ex[c] + E[0]; Ey[c] = Ey[c] + E[1]; Ez[c] = Ez[c] + E[2];
                Hx[c] = Hx[c] + H[0]; Hy[c] = Hy[c] + H[1]; Hz[c] = Hz[c] + H[2];
            });
        } else
        /* point source: cpmlfdtd.f08:3901-3906 */
        {
            const size_t c = IX3(isource, jsource, ksource);
            Ex[c] = Ex[c] + src_at(srcfn[E3_SRCX], it) * dt / e11[c];
            Ey[c] = Ey[c] + src_at(srcfn[E3_SRCY], it) * dt / e22[c];
            Ez[c] = Ez[c] + src_at(srcfn[E3_SRCZ], it) * dt / e33[c];
        }
        /* Dirichlet faces on all six fields: cpmlfdtd.f08:3912-3978 */
        double* F[6] = {Ex, Ey, Ez, Hx, Hy, Hz};
        for (int q = 0; q < 6; ++q) {
            double* f = F[q];
            for (int k = 1; k <= nz; ++k)
                for (int j = 1; j <= ny; ++j) { f[IX3(1, j, k)] = 0.0; f[IX3(nx, j, k)] = 0.0; }
            for (int k = 1; k <= nz; ++k)
                for (int i = 1; i <= nx; ++i) { f[IX3(i, 1, k)] = 0.0; f[IX3(i, ny, k)] = 0.0; }
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i) { f[IX3(i, j, 1)] = 0.0; f[IX3(i, j, nz)] = 0.0; }
        }
        memcpy(Ex_old, Ex, sizeof(double) * N);
        memcpy(Ey_old, Ey, sizeof(double) * N);
        memcpy(Ez_old, Ez, sizeof(double) * N);
        /* norm: cpmlfdtd.f08:3987-3988 */
        double velocnorm = 0.0;
#pragma omp parallel for reduction(max : velocnorm) schedule(static)
        for (size_t c = 0; c < N; ++c) {
            const double n = sqrt(Ex[c] * Ex[c] + Ey[c] * Ey[c] + Ez[c] * Ez[c]);
            velocnorm = velocnorm > n ? velocnorm : n;
        }
        if (norms) norms[step] = velocnorm;
        if (traces)
            for (int r = 0; r < nrec; ++r) {
                traces[((size_t)step * 3 + 0) * nrec + r] = Ex[rec[r]];
                traces[((size_t)step * 3 + 1) * nrec + r] = Ey[rec[r]];
                traces[((size_t)step * 3 + 2) * nrec + r] = Ez[rec[r]];
            }
        if (velocnorm > STABILITY_THRESHOLD) { free(buf); return it; }
    }
    free(buf);
    return 0;
}

