// material.cu -- material pre-pass: a material-ID image expanded into the
// padded per-cell coefficient grids the solvers read, with the boundary values
// carried into the CPML, as legacy/cpmlfdtd_cbindings.f95:60-611 does
// (permittivity_write[_c], stiffness_write, attenuation_write).
//
// The expansion is a one-off host pass over the padded grid.  The carry into
// the CPML repeats the reference's statement order exactly, because several
// statements read arrays that earlier statements of the same sweep are still
// filling in, which shapes the corner and edge values:
//   for i = 1 .. P+1 (P = CPML width):
//     rows i        <- row P+1             (low x)
//     rows nx+P-1+i <- row nx+P-1          (high x; the last interior row too)
//     cols i        <- col P+1             (low z)
//     cols nz+P-1+i <- col nz+P-1          (high z)
// with, in the permittivity pass, the reference's cross-array statements:
// sig12 is never carried to high x (its statement there writes sig13, which
// the next statement overwrites), and at low z sig12 takes sig11's column and
// sig23 takes sig33's column (cbindings:162-185).
// Grids are Fortran order (x fastest) on the padded grid (nx+2P) x (nz+2P);
// the image holds 1-based row numbers of the material table (the reference
// reads mlist(im(i,j), col)); tables are row-major [nmat][ncol] as a NumPy
// caller holds them.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <complex>
#include <string>
#include <vector>

#include "../../include/seidart_gpu.h"

extern "C" int seidart_internal_set_error(int code, const char* msg);
extern "C" int seidart_internal_write_record(const char* path, const void* data, size_t bytes);

namespace {

int merr(int code, const std::string& m) { return seidart_internal_set_error(code, m.c_str()); }

// A padded grid of T with the reference's 1-based (i, j) addressing.
template <typename T>
struct Grid {
    int NX = 0, NZ = 0;
    std::vector<T> v;
    Grid() = default;
    Grid(int nx, int nz, T fill) : NX(nx), NZ(nz), v((size_t)nx * nz, fill) {}
    T& at(int i, int j) { return v[(size_t)(i - 1) + (size_t)NX * (j - 1)]; }
    // a(dst, :) = b(src, :) and a(:, dst) = b(:, src), right side read first
    void row_from(int dst, Grid& b, int src) {
        std::vector<T> tmp(NZ);
        for (int j = 1; j <= NZ; ++j) tmp[j - 1] = b.at(src, j);
        for (int j = 1; j <= NZ; ++j) at(dst, j) = tmp[j - 1];
    }
    void col_from(int dst, Grid& b, int src) {
        std::vector<T> tmp(NX);
        for (int i = 1; i <= NX; ++i) tmp[i - 1] = b.at(i, src);
        for (int i = 1; i <= NX; ++i) at(i, dst) = tmp[i - 1];
    }
};

struct Image {
    const int* im;
    int nx, nz, nmat;
    // material row (0-based) of interior cell (ii, jj), 1-based
    int row(int ii, int jj) const { return im[(size_t)(ii - 1) + (size_t)nx * (jj - 1)] - 1; }
};

int check_inputs(const int* im, int nx, int nz, const void* table, int nmat, int ncol, int need, int npml) {
    if (!im || !table || nx < 1 || nz < 1 || nmat < 1 || npml < 0)
        return merr(SEIDART_ERR_ARG, "material pre-pass: bad sizes or NULL arrays");
    if (ncol < need) {
        char m[128];
        snprintf(m, sizeof m, "material table needs at least %d columns, got %d", need, ncol);
        return merr(SEIDART_ERR_ARG, m);
    }
    if (nx < 2 || nz < 2)
        return merr(SEIDART_ERR_ARG, "material pre-pass: the CPML carry needs nx, nz >= 2");
    for (size_t q = 0; q < (size_t)nx * nz; ++q)
        if (im[q] < 1 || im[q] > nmat) {
            char m[160];
            snprintf(m, sizeof m, "material image value %d at cell %zu is not a table row (1..%d)", im[q], q, nmat);
            return merr(SEIDART_ERR_ARG, m);
        }
    return SEIDART_OK;
}

// interior fill: g[a](i, j) = table(im(i-P, j-P), col0 + a)  (1-based columns)
template <typename T, typename Get>
void fill_interior(std::vector<Grid<T>>& g, const Image& I, int P, int col0, Get get) {
    for (size_t a = 0; a < g.size(); ++a)
        for (int j = P + 1; j <= I.nz + P; ++j)
            for (int i = P + 1; i <= I.nx + P; ++i) g[a].at(i, j) = get(I.row(i - P, j - P), col0 + (int)a);
}

// the plain carry of one array into the CPML (stiffness arrays, eps arrays)
template <typename T>
void carry_rows_lo(Grid<T>& a, int i, int P) { a.row_from(i, a, P + 1); }
template <typename T>
void carry_rows_hi(Grid<T>& a, int i, int P, int nx) { a.row_from(nx + P - 1 + i, a, nx + P - 1); }
template <typename T>
void carry_cols_lo(Grid<T>& a, int i, int P) { a.col_from(i, a, P + 1); }
template <typename T>
void carry_cols_hi(Grid<T>& a, int i, int P, int nz) { a.col_from(nz + P - 1 + i, a, nz + P - 1); }

// permittivity carry (cbindings:119-185): eps = 6 arrays in the order eps11 22
// 33 12 13 23 of the reference's statements, sig likewise sig11 22 33 12 13 23
template <typename TE>
void carry_permittivity(std::vector<Grid<TE>>& eps, std::vector<Grid<double>>& sig, int P, int nx, int nz) {
    // statement order of the reference: 11 22 33 12 13 23
    const int ord[6] = {0, 3, 5, 1, 2, 4};  // positions of 11,22,33,12,13,23 in our 11 12 13 22 23 33 order
    Grid<double>&s11 = sig[0], &s12 = sig[1], &s13 = sig[2], &s22 = sig[3], &s23 = sig[4], &s33 = sig[5];
    for (int i = 1; i <= P + 1; ++i) {
        for (int q : ord) carry_rows_lo(eps[q], i, P);
        for (int q : ord) carry_rows_hi(eps[q], i, P, nx);
        for (int q : ord) carry_rows_lo(sig[q], i, P);
        // high x: sig12's statement writes sig13 (overwritten next): sig12 is not carried
        const int hi = nx + P - 1 + i, src = nx + P - 1;
        s11.row_from(hi, s11, src);
        s22.row_from(hi, s22, src);
        s33.row_from(hi, s33, src);
        s13.row_from(hi, s12, src);
        s13.row_from(hi, s13, src);
        s23.row_from(hi, s23, src);
        for (int q : ord) carry_cols_lo(eps[q], i, P);
        for (int q : ord) carry_cols_hi(eps[q], i, P, nz);
        // low z: sig12 <- sig11's column, sig23 <- sig33's column
        s11.col_from(i, s11, P + 1);
        s22.col_from(i, s22, P + 1);
        s33.col_from(i, s33, P + 1);
        s12.col_from(i, s11, P + 1);
        s13.col_from(i, s13, P + 1);
        s23.col_from(i, s33, P + 1);
        for (int q : ord) carry_cols_hi(sig[q], i, P, nz);
    }
}

template <typename T>
void copy_out(const std::vector<Grid<T>>& g, double* const* out, size_t first) {
    for (size_t a = 0; a < g.size(); ++a)
        if (out[first + a]) memcpy(out[first + a], g[a].v.data(), g[a].v.size() * sizeof(T));
}

int stiffness(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml, const double* gradient,
              std::vector<Grid<double>>& g) {
    int rc = check_inputs(im, nx, nz, mlist, nmat, ncol, 23, npml);
    if (rc != SEIDART_OK) return rc;
    const int P = npml, NX = nx + 2 * P, NZ = nz + 2 * P;
    g.assign(22, Grid<double>(NX, NZ, 0.0));
    const Image I{im, nx, nz, nmat};
    fill_interior(g, I, P, 2, [&](int r, int col) { return mlist[(size_t)r * ncol + (col - 1)]; });
    if (gradient)  // rho(interior) = rho(interior) * gradient  (cbindings:433-434)
        for (int j = P + 1; j <= nz + P; ++j)
            for (int i = P + 1; i <= nx + P; ++i)
                g[21].at(i, j) = g[21].at(i, j) * gradient[(size_t)(i - P - 1) + (size_t)nx * (j - P - 1)];
    for (int i = 1; i <= P + 1; ++i) {
        for (auto& a : g) carry_rows_lo(a, i, P);
        for (auto& a : g) carry_rows_hi(a, i, P, nx);
        for (auto& a : g) carry_cols_lo(a, i, P);
        for (auto& a : g) carry_cols_hi(a, i, P, nz);
    }
    return SEIDART_OK;
}

int permittivity(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                 std::vector<Grid<double>>& eps, std::vector<Grid<double>>& sig) {
    int rc = check_inputs(im, nx, nz, mlist, nmat, ncol, 13, npml);
    if (rc != SEIDART_OK) return rc;
    const int P = npml, NX = nx + 2 * P, NZ = nz + 2 * P;
    eps.assign(6, Grid<double>(NX, NZ, 0.0));
    sig.assign(6, Grid<double>(NX, NZ, 0.0));
    const Image I{im, nx, nz, nmat};
    auto get = [&](int r, int col) { return mlist[(size_t)r * ncol + (col - 1)]; };
    fill_interior(eps, I, P, 2, get);
    fill_interior(sig, I, P, 8, get);
    carry_permittivity(eps, sig, P, nx, nz);
    return SEIDART_OK;
}

using cplx = std::complex<double>;
int permittivity_c(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                   std::vector<Grid<cplx>>& eps, std::vector<Grid<double>>& sig) {
    int rc = check_inputs(im, nx, nz, mlist, nmat, ncol, 13, npml);
    if (rc != SEIDART_OK) return rc;
    const int P = npml, NX = nx + 2 * P, NZ = nz + 2 * P;
    eps.assign(6, Grid<cplx>(NX, NZ, cplx(0.0, 0.0)));
    sig.assign(6, Grid<double>(NX, NZ, 0.0));
    const Image I{im, nx, nz, nmat};
    auto getc = [&](int r, int col) {
        const size_t q = ((size_t)r * ncol + (col - 1)) * 2;
        return cplx(mlist[q], mlist[q + 1]);
    };
    fill_interior(eps, I, P, 2, getc);
    // |z| as gfortran's abs(complex) computes it: the C library's hypot (cbindings:264-269)
    fill_interior(sig, I, P, 8, [&](int r, int col) {
        const cplx z = getc(r, col);
        return hypot(z.real(), z.imag());
    });
    carry_permittivity(eps, sig, P, nx, nz);
    return SEIDART_OK;
}

int attenuation(const int* im, int nx, int nz, const double* alist, int nmat, int ncol, int npml, double cpmlvalue,
                std::vector<Grid<double>>& g) {
    int rc = check_inputs(im, nx, nz, alist, nmat, ncol, 3, npml);
    if (rc != SEIDART_OK) return rc;
    const int P = npml;
    g.assign(3, Grid<double>(nx + 2 * P, nz + 2 * P, cpmlvalue));  // no carry: the CPML keeps cpmlvalue
    fill_interior(g, Image{im, nx, nz, nmat}, P, 1, [&](int r, int col) { return alist[(size_t)r * ncol + (col - 1)]; });
    return SEIDART_OK;
}

template <typename T>
int write_all(const char* dir, const char* const* names, const std::vector<Grid<T>>& g) {
    const std::string d = (dir && *dir) ? std::string(dir) + "/" : std::string();
    for (size_t a = 0; a < g.size(); ++a) {
        const int rc = seidart_internal_write_record((d + names[a]).c_str(), g[a].v.data(), g[a].v.size() * sizeof(T));
        if (rc != SEIDART_OK) return rc;
    }
    return SEIDART_OK;
}

const char* kStiffNames[22] = {"c11.dat", "c12.dat", "c13.dat", "c14.dat", "c15.dat", "c16.dat", "c22.dat", "c23.dat",
                               "c24.dat", "c25.dat", "c26.dat", "c33.dat", "c34.dat", "c35.dat", "c36.dat", "c44.dat",
                               "c45.dat", "c46.dat", "c55.dat", "c56.dat", "c66.dat", "rho.dat"};
const char* kEpsNames[6] = {"eps11.dat", "eps12.dat", "eps13.dat", "eps22.dat", "eps23.dat", "eps33.dat"};
const char* kSigNames[6] = {"sig11.dat", "sig12.dat", "sig13.dat", "sig22.dat", "sig23.dat", "sig33.dat"};
const char* kGamNames[3] = {"gamma_x.dat", "gamma_y.dat", "gamma_z.dat"};

}  // namespace

extern "C" {

int seidart_stiffness_arrays(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                             const double* gradient, double* const* out) {
    std::vector<Grid<double>> g;
    const int rc = stiffness(im, nx, nz, mlist, nmat, ncol, npml, gradient, g);
    if (rc == SEIDART_OK && out) copy_out(g, out, 0);
    return rc;
}

int seidart_stiffness_write(const char* dir, const int* im, int nx, int nz, const double* mlist, int nmat, int ncol,
                            int npml, const double* gradient) {
    std::vector<Grid<double>> g;
    const int rc = stiffness(im, nx, nz, mlist, nmat, ncol, npml, gradient, g);
    return rc == SEIDART_OK ? write_all(dir, kStiffNames, g) : rc;
}

int seidart_permittivity_arrays(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                                double* const* out) {
    std::vector<Grid<double>> eps, sig;
    const int rc = permittivity(im, nx, nz, mlist, nmat, ncol, npml, eps, sig);
    if (rc == SEIDART_OK && out) {
        copy_out(eps, out, 0);
        copy_out(sig, out, 6);
    }
    return rc;
}

int seidart_permittivity_write(const char* dir, const int* im, int nx, int nz, const double* mlist, int nmat,
                               int ncol, int npml) {
    std::vector<Grid<double>> eps, sig;
    int rc = permittivity(im, nx, nz, mlist, nmat, ncol, npml, eps, sig);
    if (rc == SEIDART_OK) rc = write_all(dir, kEpsNames, eps);
    if (rc == SEIDART_OK) rc = write_all(dir, kSigNames, sig);
    return rc;
}

int seidart_permittivity_arrays_c(const int* im, int nx, int nz, const double* mlist_c, int nmat, int ncol, int npml,
                                  double* const* out) {
    std::vector<Grid<cplx>> eps;
    std::vector<Grid<double>> sig;
    const int rc = permittivity_c(im, nx, nz, mlist_c, nmat, ncol, npml, eps, sig);
    if (rc == SEIDART_OK && out) {
        for (size_t a = 0; a < eps.size(); ++a)
            if (out[a]) memcpy(out[a], eps[a].v.data(), eps[a].v.size() * sizeof(cplx));
        copy_out(sig, out, 6);
    }
    return rc;
}

int seidart_permittivity_write_c(const char* dir, const int* im, int nx, int nz, const double* mlist_c, int nmat,
                                 int ncol, int npml) {
    std::vector<Grid<cplx>> eps;
    std::vector<Grid<double>> sig;
    int rc = permittivity_c(im, nx, nz, mlist_c, nmat, ncol, npml, eps, sig);
    if (rc == SEIDART_OK) rc = write_all(dir, kEpsNames, eps);
    if (rc == SEIDART_OK) rc = write_all(dir, kSigNames, sig);
    return rc;
}

int seidart_attenuation_arrays(const int* im, int nx, int nz, const double* alist, int nmat, int ncol, int npml,
                               double cpmlvalue, double* const* out) {
    std::vector<Grid<double>> g;
    const int rc = attenuation(im, nx, nz, alist, nmat, ncol, npml, cpmlvalue, g);
    if (rc == SEIDART_OK && out) copy_out(g, out, 0);
    return rc;
}

int seidart_attenuation_write(const char* dir, const int* im, int nx, int nz, const double* alist, int nmat, int ncol,
                              int npml, double cpmlvalue) {
    std::vector<Grid<double>> g;
    const int rc = attenuation(im, nx, nz, alist, nmat, ncol, npml, cpmlvalue, g);
    return rc == SEIDART_OK ? write_all(dir, kGamNames, g) : rc;
}

}  // extern "C"
