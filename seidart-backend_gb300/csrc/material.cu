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
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
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

// ------------------------------------------------------------ device pass
// The same expansion as device kernels writing the padded FP64 grids in
// device memory: one fill kernel (interior from the table, the CPML at its
// initial value), then per carry iteration i = 1..P+1 a row phase and a
// column phase.  Within a phase every statement reads a row (column) that no
// statement of the phase writes, except no-op self copies (i = P+1), so the
// statements of a phase run in parallel and the phases keep the reference's
// order.  Per-material values that need arithmetic (|eps| for complex
// permittivity) are formed on the host over the small table, so the device
// result equals the host pass bit for bit.
enum { K_PLAIN = 0, K_SIG12 = 1, K_SIG13 = 2, K_SIG23 = 3 };  // carry kinds (permittivity quirks)

struct DevPass {
    double* out[22];  // device grids (complex ones as interleaved pairs)
    int kind[22];     // K_* carry role of each array
    int narr;
    int cplx[22];     // 1: complex grid (two doubles per cell)
    int NX, NZ, P, nx, nz;
};

// interior fill: out[a](i, j) = tab[row(im)][a] (complex: two doubles), and
// optionally times the density gradient; CPML cells get `edge`
__global__ void mat_fill(DevPass D, const int* __restrict__ im, const double* __restrict__ tab, int tstride,
                         const double* __restrict__ grad, int grad_arr, double edge) {
    const size_t cells = (size_t)D.NX * D.NZ;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < cells * D.narr;
         q += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / cells);
        const size_t c = q - (size_t)a * cells;
        const int i = (int)(c % D.NX), j = (int)(c / D.NX);  // 0-based padded
        const int ii = i - D.P, jj = j - D.P;
        const bool in = ii >= 0 && ii < D.nx && jj >= 0 && jj < D.nz;
        if (D.cplx[a]) {
            double re = edge, imv = 0.0;
            if (in) {
                const int r = im[(size_t)ii + (size_t)D.nx * jj] - 1;
                re = tab[(size_t)r * tstride + 2 * a];
                imv = tab[(size_t)r * tstride + 2 * a + 1];
            }
            D.out[a][2 * c] = re;
            D.out[a][2 * c + 1] = imv;
        } else {
            double v = edge;
            if (in) {
                const int r = im[(size_t)ii + (size_t)D.nx * jj] - 1;
                v = tab[(size_t)r * tstride + (D.cplx[0] ? 2 * a : a)];
                if (grad && a == grad_arr) v = v * grad[(size_t)ii + (size_t)D.nx * jj];
            }
            D.out[a][c] = v;
        }
    }
}

__device__ __forceinline__ void cp_cell(const DevPass& D, int dst_a, size_t dc, int src_a, size_t sc) {
    if (D.cplx[dst_a]) {
        const double re = D.out[src_a][2 * sc], imv = D.out[src_a][2 * sc + 1];
        D.out[dst_a][2 * dc] = re;
        D.out[dst_a][2 * dc + 1] = imv;
    } else {
        D.out[dst_a][dc] = D.out[src_a][sc];
    }
}

// row phase of iteration i (1-based): rows i <- P+1 and nx+P-1+i <- nx+P-1;
// the sig12 array is not carried to high x (its statement writes sig13,
// which the sig13 statement overwrites with its own carry)
__global__ void mat_rows(DevPass D, int i) {
    const int NX = D.NX, NZ = D.NZ;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < (size_t)D.narr * NZ * 2;
         q += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / (2 * (size_t)NZ));
        const int r = (int)(q - (size_t)a * 2 * NZ);
        const int j = r % NZ, hi = r / NZ;  // 0-based column, 0 low / 1 high
        const int dst = hi ? (D.nx + D.P - 1 + i) - 1 : i - 1, src = hi ? (D.nx + D.P - 1) - 1 : D.P;
        if (dst == src) continue;
        if (hi && D.kind[a] == K_SIG12) continue;
        cp_cell(D, a, (size_t)dst + (size_t)NX * j, a, (size_t)src + (size_t)NX * j);
    }
}

// column phase of iteration i: cols i <- P+1 and nz+P-1+i <- nz+P-1; at
// low z sig12 takes sig11's column and sig23 takes sig33's column
__global__ void mat_cols(DevPass D, int i, int sig11, int sig33) {
    const int NX = D.NX;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < (size_t)D.narr * NX * 2;
         q += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / (2 * (size_t)NX));
        const int r = (int)(q - (size_t)a * 2 * NX);
        const int row = r % NX, hi = r / NX;
        const int dst = hi ? (D.nz + D.P - 1 + i) - 1 : i - 1, src = hi ? (D.nz + D.P - 1) - 1 : D.P;
        int from = a;
        if (!hi && D.kind[a] == K_SIG12) from = sig11;
        if (!hi && D.kind[a] == K_SIG23) from = sig33;
        if (dst == src && from == a) continue;
        cp_cell(D, a, (size_t)row + (size_t)NX * dst, from, (size_t)row + (size_t)NX * src);
    }
}

// Upload the image (and the gradient), run fill + carry on `st`, free the
// scratch.  tab: host table already reduced to the output columns (tstride
// doubles per material row).  carry = false: attenuation (the CPML keeps
// `edge`).
int run_dev_pass(DevPass D, const int* im, const std::vector<double>& tab, int tstride, const double* grad,
                 int grad_arr, double edge, bool carry, int sig11, int sig33, cudaStream_t st) {
    int* dim = nullptr;
    double* dtab = nullptr;
    double* dgrad = nullptr;
    const size_t ncell = (size_t)D.nx * D.nz;
    auto fail = [&](const char* what) {
        cudaGetLastError();
        if (dim) cudaFree(dim);
        if (dtab) cudaFree(dtab);
        if (dgrad) cudaFree(dgrad);
        return merr(SEIDART_ERR_CUDA, std::string("device material pre-pass: ") + what);
    };
    if (cudaMalloc((void**)&dim, ncell * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void**)&dtab, tab.size() * sizeof(double)) != cudaSuccess ||
        (grad && cudaMalloc((void**)&dgrad, ncell * sizeof(double)) != cudaSuccess))
        return fail("scratch allocation");
    if (cudaMemcpyAsync(dim, im, ncell * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (grad && cudaMemcpyAsync(dgrad, grad, ncell * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess))
        return fail("upload");
    mat_fill<<<4 * 152, 256, 0, st>>>(D, dim, dtab, tstride, dgrad, grad_arr, edge);
    if (carry)
        for (int i = 1; i <= D.P + 1; ++i) {
            mat_rows<<<(unsigned)std::min<size_t>(4 * 152, ((size_t)D.narr * D.NZ * 2 + 255) / 256), 256, 0, st>>>(D, i);
            mat_cols<<<(unsigned)std::min<size_t>(4 * 152, ((size_t)D.narr * D.NX * 2 + 255) / 256), 256, 0, st>>>(
                D, i, sig11, sig33);
        }
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) return fail("kernels");
    cudaFree(dim);
    cudaFree(dtab);
    if (dgrad) cudaFree(dgrad);
    return SEIDART_OK;
}

// host table reduced to the output columns: row r holds `count` values
// starting at 1-based column col0 (complex tables: interleaved pairs)
std::vector<double> table_cols(const double* t, int nmat, int ncol, int col0, int count, bool cplx) {
    const int w = cplx ? 2 : 1;
    std::vector<double> out((size_t)nmat * count * w);
    for (int r = 0; r < nmat; ++r)
        for (int a = 0; a < count; ++a)
            for (int c = 0; c < w; ++c) out[((size_t)r * count + a) * w + c] = t[((size_t)r * ncol + col0 - 1 + a) * w + c];
    return out;
}

DevPass dev_pass(double* const* out, int narr, int nx, int nz, int P) {
    DevPass D{};
    D.narr = narr;
    D.nx = nx; D.nz = nz; D.P = P;
    D.NX = nx + 2 * P; D.NZ = nz + 2 * P;
    for (int a = 0; a < narr; ++a) { D.out[a] = out[a]; D.kind[a] = K_PLAIN; D.cplx[a] = 0; }
    return D;
}

}  // namespace

extern "C" {

int seidart_stiffness_arrays_dev(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                                 const double* gradient, double* const* dev_out, void* stream) {
    int rc = check_inputs(im, nx, nz, mlist, nmat, ncol, 23, npml);
    if (rc != SEIDART_OK) return rc;
    if (!dev_out) return merr(SEIDART_ERR_ARG, "dev_out must not be NULL");
    for (int a = 0; a < 22; ++a)
        if (!dev_out[a]) return merr(SEIDART_ERR_ARG, "every stiffness output grid is needed (the carry reads them)");
    DevPass D = dev_pass(dev_out, 22, nx, nz, npml);
    return run_dev_pass(D, im, table_cols(mlist, nmat, ncol, 2, 22, false), 22, gradient, 21, 0.0, true, -1, -1,
                        (cudaStream_t)stream);
}

int seidart_permittivity_arrays_dev(const int* im, int nx, int nz, const double* mlist, int nmat, int ncol, int npml,
                                    double* const* dev_out, void* stream) {
    int rc = check_inputs(im, nx, nz, mlist, nmat, ncol, 13, npml);
    if (rc != SEIDART_OK) return rc;
    if (!dev_out) return merr(SEIDART_ERR_ARG, "dev_out must not be NULL");
    for (int a = 0; a < 12; ++a)
        if (!dev_out[a]) return merr(SEIDART_ERR_ARG, "every permittivity output grid is needed (the carry reads them)");
    // eps11 12 13 22 23 33 (cols 2..7), sig11 12 13 22 23 33 (cols 8..13)
    DevPass D = dev_pass(dev_out, 12, nx, nz, npml);
    D.kind[7] = K_SIG12; D.kind[8] = K_SIG13; D.kind[10] = K_SIG23;
    return run_dev_pass(D, im, table_cols(mlist, nmat, ncol, 2, 12, false), 12, nullptr, -1, 0.0, true, 6, 11,
                        (cudaStream_t)stream);
}

int seidart_permittivity_arrays_c_dev(const int* im, int nx, int nz, const double* mlist_c, int nmat, int ncol,
                                      int npml, double* const* dev_out, void* stream) {
    int rc = check_inputs(im, nx, nz, mlist_c, nmat, ncol, 13, npml);
    if (rc != SEIDART_OK) return rc;
    if (!dev_out) return merr(SEIDART_ERR_ARG, "dev_out must not be NULL");
    for (int a = 0; a < 12; ++a)
        if (!dev_out[a]) return merr(SEIDART_ERR_ARG, "every permittivity output grid is needed (the carry reads them)");
    // complex eps (interleaved pairs) and sigma = |table value| formed here,
    // with the C library's hypot as the host pass uses; table rows of 12
    // complex slots, the sigma slots holding (|z|, 0)
    std::vector<double> tab = table_cols(mlist_c, nmat, ncol, 2, 12, true);
    for (int r = 0; r < nmat; ++r)
        for (int a = 6; a < 12; ++a) {
            double* z = &tab[((size_t)r * 12 + a) * 2];
            z[0] = hypot(z[0], z[1]);
            z[1] = 0.0;
        }
    DevPass D = dev_pass(dev_out, 12, nx, nz, npml);
    for (int a = 0; a < 6; ++a) D.cplx[a] = 1;
    D.kind[7] = K_SIG12; D.kind[8] = K_SIG13; D.kind[10] = K_SIG23;
    return run_dev_pass(D, im, tab, 24, nullptr, -1, 0.0, true, 6, 11, (cudaStream_t)stream);
}

int seidart_attenuation_arrays_dev(const int* im, int nx, int nz, const double* alist, int nmat, int ncol, int npml,
                                   double cpmlvalue, double* const* dev_out, void* stream) {
    int rc = check_inputs(im, nx, nz, alist, nmat, ncol, 3, npml);
    if (rc != SEIDART_OK) return rc;
    if (!dev_out) return merr(SEIDART_ERR_ARG, "dev_out must not be NULL");
    for (int a = 0; a < 3; ++a)
        if (!dev_out[a]) return merr(SEIDART_ERR_ARG, "every attenuation output grid is needed");
    DevPass D = dev_pass(dev_out, 3, nx, nz, npml);
    return run_dev_pass(D, im, table_cols(alist, nmat, ncol, 1, 3, false), 3, nullptr, -1, cpmlvalue, false, -1, -1,
                        (cudaStream_t)stream);
}

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
