// planewave.cu -- plane-wave sources: set-up on the host and injection
// kernels on the device.
//
// A plane-wave source (source_type "pw", and for the elastic solvers also
// "pws"/"pw_s"/"pw-s" and the P-wave forms "pwp"/"pw_p"/"pw-p") injects
// the analytic field of a plane wave on up to three faces of the interior
// box after every velocity / E update (src/fortran/plane_wave_source.f08,
// cpmlfdtd.f08:186-227 and :452-512 seismic2, :802-834 and :1207-1260
// seismic25, :1548-1606 and :2133-2203 seismic3, :2436-2476 and :2626-2673
// electromag2, :3523-3578 and :3833-3900 electromag3):
//   p = R k0, ehat = transverse part of R e0 (R = Ry(xz) Rz(xy) Rx(yz),
//   k0 = z, e0 = x; ehat = p for a P wave), one face per non-zero component
//   of p (the face the wave enters through), r0 on that face, and at time
//   t = it dt, per face cell r:  tau = t - p.(r - r0)/v,  s = amp w(tau),
//   w = gaus0|gaus1|gaus2 (Gaussian and its derivatives, t0 = 1.5/f0).
//   Elastic: v += s ehat, sigma += C : strain, strain = -(s/v) sym(ehat p);
//   v = sqrt(max eigenvalue of the Mandel stiffness over the grid / min rho).
//   EM: E += s ehat, H += (s/eta) (p x ehat)/|p x ehat|; v = c/sqrt(eps_min),
//   eta = sqrt(mu0/(eps0 eps_min)), eps_min the smallest permittivity
//   eigenvalue over the grid.
// The eigenvalues (LAPACK dsyev in the reference, tensor_operations.f08)
// come from a cyclic Jacobi iteration in FP64 here, over the distinct
// material tuples of the grid only.
//
// Device side: one launch per face in x, y, z order (cells where faces meet
// receive the adds in the reference's order), then one launch that takes the
// max-norms of all face cells; the solver's velocity / E kernels leave those
// cells out of their norms.  Fields the reference zeroes on the outer faces
// after the injection (velocities, E, H) are not touched there; stresses are.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/seidart_gpu.h"
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr double kPi = 3.1415926535897932384626433832795;

// ------------------------------------------------------------------ host
// Eigenvalues of a symmetric n x n matrix (row-major, n <= 6) by cyclic
// Jacobi rotations (Golub & Van Loan, Matrix Computations, sec. 8.5),
// returned in ascending order.
void jacobi_eigenvalues(int n, double* a, double* lam) {
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i) {
            diag += a[i * n + i] * a[i * n + i];
            for (int j = i + 1; j < n; ++j) off += a[i * n + j] * a[i * n + j];
        }
        if (off == 0.0 || off <= 1e-36 * diag) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a[p * n + q];
                if (apq == 0.0) continue;
                const double theta = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {  // columns p, q
                    const double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // rows p, q
                    const double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                a[p * n + q] = a[q * n + p] = 0.0;
            }
    }
    for (int i = 0; i < n; ++i) lam[i] = a[i * n + i];
    std::sort(lam, lam + n);
}

// distinct tuples of `k` grids over N cells -> f(tuple), combined by `keep`
template <typename F, typename K>
double over_tuples(size_t N, int k, const double* const* g, double init, F f, K keep) {
    struct H {
        size_t operator()(const std::string& s) const { return std::hash<std::string>()(s); }
    };
    std::unordered_map<std::string, double, H> seen;
    double acc = init;
    std::string key(k * sizeof(double), '\0');
    std::vector<double> t(k);
    for (size_t c = 0; c < N; ++c) {
        for (int q = 0; q < k; ++q) t[q] = g[q][c];
        memcpy(&key[0], t.data(), k * sizeof(double));
        auto it = seen.find(key);
        double v;
        if (it != seen.end()) {
            v = it->second;
        } else {
            v = f(t.data());
            seen.emplace(key, v);
        }
        acc = keep(acc, v);
    }
    return acc;
}

// largest eigenvalue of the Mandel form of a 6x6 Voigt stiffness (upper
// triangle in C21 order; eigen4, tensor_operations.f08:56-132)
double mandel_max_eig(const double* c21) {
    double a[36];
    int q = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) a[i * 6 + j] = a[j * 6 + i] = c21[q++];
    const double s[6] = {1.0, 1.0, 1.0, sqrt(2.0), sqrt(2.0), sqrt(2.0)};
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) a[i * 6 + j] *= s[i] * s[j];
    double lam[6];
    jacobi_eigenvalues(6, a, lam);
    return lam[5];
}

void rot(double xz, double xy, double yz, double R[3][3]) {
    // rotmat (plane_wave_source.f08:76-108): R = Ry(xz) Rz(xy) Rx(yz), degrees.
    // The reference builds each factor with reshape, which fills columns, so
    // the factors below (row-major) are the transposes of its listings.
    const double d = kPi / 180.0;
    const double cx = cos(d * yz), cy = cos(d * xz), cz = cos(d * xy);
    const double sx = sin(d * yz), sy = sin(d * xz), sz = sin(d * xy);
    const double Rx[3][3] = {{1, 0, 0}, {0, cx, sx}, {0, -sx, cx}};
    const double Ry[3][3] = {{cy, 0, -sy}, {0, 1, 0}, {sy, 0, cy}};
    const double Rz[3][3] = {{cz, sz, 0}, {-sz, cz, 0}, {0, 0, 1}};
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T[i][j] = 0.0;
            for (int k = 0; k < 3; ++k) T[i][j] += Rz[i][k] * Rx[k][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            R[i][j] = 0.0;
            for (int k = 0; k < 3; ++k) R[i][j] += Ry[i][k] * T[k][j];
        }
}

double norm3(const double* v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// direction_polarization_vector (plane_wave_source.f08:110-139)
void direction(double xz, double xy, double yz, double* p, double* e) {
    double R[3][3];
    rot(xz, xy, yz, R);
    for (int i = 0; i < 3; ++i) p[i] = R[i][2];  // R k0, k0 = z
    double n = norm3(p);
    if (n > 0.0)
        for (int i = 0; i < 3; ++i) p[i] /= n;
    double t[3] = {R[0][0], R[1][0], R[2][0]};  // R e0, e0 = x
    double d = t[0] * p[0] + t[1] * p[1] + t[2] * p[2];
    for (int i = 0; i < 3; ++i) t[i] -= d * p[i];
    n = norm3(t);
    if (n > 0.0) {
        for (int i = 0; i < 3; ++i) e[i] = t[i] / n;
        return;
    }
    t[0] = fabs(p[0]) < 0.9 ? 1.0 : 0.0;
    t[1] = fabs(p[0]) < 0.9 ? 0.0 : 1.0;
    t[2] = 0.0;
    d = t[0] * p[0] + t[1] * p[1] + t[2] * p[2];
    for (int i = 0; i < 3; ++i) t[i] -= d * p[i];
    n = norm3(t);
    for (int i = 0; i < 3; ++i) e[i] = n > 0.0 ? t[i] / n : 0.0;
}

// ---------------------------------------------------------------- device
// Fields touched by the injection of one family.
template <typename T>
struct PwFields {
    T* v[3];      // velocities or E (NULL: component absent); complex interleaved when cplx
    T* s[6];      // stresses sxx syy szz syz sxz sxy (seismic; NULL absent)
    T* h[3];      // H components (EM; NULL absent)
    const T* C[21];  // stiffness (C21 order; NULL absent)
    int cplx;     // 2.5D: complex interleaved fields, the adds go to the real part
    int nx, ny, nz;
    int stress_tmp;  // 2.5D: stress adds summed from zero first (tmp_s* of cpmlfdtd.f08:1224-1236)
};

__device__ __forceinline__ double pw_wavelet(const PwDev& pw, double tau) {
    // wavelet (plane_wave_source.f08:141-161)
    const double t0 = 1.5 / pw.f0;
    const double a = kPi * pw.f0 * (tau - t0);
    const double g = exp(-a * a);
    if (pw.wavelet == 1) return -2.0 * a * g;
    if (pw.wavelet == 2) return (1.0 - 2.0 * a * a) * g;
    return g;
}

// 0-based cell of thread q on face f, or false when q is past its end
__device__ __forceinline__ bool face_cell(const PwFace& f, long long q, int& i, int& j, int& k) {
    const int n0 = f.hi[0] - f.lo[0] + 1, n1 = f.hi[1] - f.lo[1] + 1, n2 = f.hi[2] - f.lo[2] + 1;
    if (q >= (long long)n0 * n1 * n2) return false;
    i = f.lo[0] + (int)(q % n0);
    j = f.lo[1] + (int)((q / n0) % n1);
    k = f.lo[2] + (int)(q / ((long long)n0 * n1));
    return true;
}

template <typename T>
__global__ void pw_inject(PwDev pw, PwFields<T> F, int face, StepInfo si) {
    const PwFace& f = pw.face[face];
    int i, j, k;
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_cell(f, q, i, j, k)) return;
    const int it = *si.step;
    const double t = it * pw.dt;
    // r: the face's location on its axis, (index + 1) h on the others (2D: y = 0)
    double r[3];
    const int idx[3] = {i, j, k};
    for (int d = 0; d < 3; ++d) r[d] = d == f.axis ? pw.loc[d] : (double)(idx[d] + 1) * pw.h[d];
    if (F.ny == 1) r[1] = 0.0;
    const double tau = t - (pw.p[0] * (r[0] - pw.r0[0]) + pw.p[1] * (r[1] - pw.r0[1]) + pw.p[2] * (r[2] - pw.r0[2])) / pw.v;
    const double s = pw.amp * pw_wavelet(pw, tau);
    const size_t c = (size_t)i + (size_t)F.nx * ((size_t)j + (size_t)F.ny * k);
    const size_t cc = F.cplx ? 2 * c : c;
    const bool outer = i == 0 || i == F.nx - 1 || k == 0 || k == F.nz - 1 || (F.ny > 1 && (j == 0 || j == F.ny - 1));
    if (!outer) {
        for (int d = 0; d < 3; ++d)
            if (F.v[d]) F.v[d][cc] = (T)((double)F.v[d][cc] + s * pw.ehat[d]);
        for (int d = 0; d < 3; ++d)
            if (F.h[d]) F.h[d][cc] = (T)((double)F.h[d][cc] + (s / pw.eta) * pw.hhat[d]);
    }
    if (!F.s[0] && !F.s[2]) return;
    const double sc = -s / pw.v;
    const double* e = pw.ehat;
    const double* p = pw.p;
    const double st[6] = {sc * e[0] * p[0], sc * e[1] * p[1], sc * e[2] * p[2], sc * (e[1] * p[2] + e[2] * p[1]),
                          sc * (e[0] * p[2] + e[2] * p[0]), sc * (e[0] * p[1] + e[1] * p[0])};
    // C21 index of the symmetric entry (row a, column b), 0-based Voigt indices
    auto cij = [&](int a, int b) -> double {
        const int lo = a < b ? a : b, hi = a < b ? b : a;
        const int q21 = lo * 6 - lo * (lo - 1) / 2 + (hi - lo);
        return F.C[q21] ? (double)F.C[q21][c] : 0.0;
    };
    // add_plane_wave_stress (cpmlfdtd.f08:16-50); 2D seismic2 uses the
    // xx / zz / xz rows with strain 1, 3, 5 only (:477-485)
    const int row_of[6] = {0, 1, 2, 3, 4, 5};  // sxx syy szz syz sxz sxy  <->  Voigt rows 1..6
    for (int w = 0; w < 6; ++w) {
        T* sg = F.s[w];
        if (!sg) continue;
        const int a = row_of[w];
        if (F.ny == 1 && !F.cplx) {  // seismic2
            const double add1 = cij(a, 0) * st[0], add3 = cij(a, 2) * st[2], add5 = cij(a, 4) * st[4];
            sg[cc] = (T)((double)sg[cc] + add1 + add3 + add5);
        } else if (F.stress_tmp) {
            double tmp = 0.0;
            for (int b = 0; b < 6; ++b) tmp = tmp + cij(a, b) * st[b];
            sg[cc] = (T)((double)sg[cc] + tmp);
        } else {
            double acc = (double)sg[cc];
            for (int b = 0; b < 6; ++b) acc = acc + cij(a, b) * st[b];
            sg[cc] = (T)acc;
        }
    }
}

// max-norms of every face cell after all faces' adds
template <typename T>
__global__ void pw_norms(PwDev pw, PwFields<T> F, StepInfo si, double* vnorm, double* snorm) {
    const int face = blockIdx.y;
    if (face >= pw.nface) return;
    int i, j, k;
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double vn = 0.0, sn = 0.0;
    if (face_cell(pw.face[face], q, i, j, k)) {
        const size_t c = (size_t)i + (size_t)F.nx * ((size_t)j + (size_t)F.ny * k);
        double acc = 0.0;
        for (int d = 0; d < 3; ++d)
            if (F.v[d]) {
                if (F.cplx) {
                    const double re = F.v[d][2 * c], im = F.v[d][2 * c + 1];
                    acc += re * re + im * im;
                } else {
                    const double x = F.v[d][c];
                    acc += x * x;
                }
            }
        vn = sqrt(acc);
        if (snorm) {
            const double s1 = F.s[0][c], s2 = F.s[1][c], s3 = F.s[2][c];
            const double s4 = F.s[5][c], s5 = F.s[3][c], s6 = F.s[4][c];  // sxy syz sxz
            sn = sqrt(s1 * s1 + s2 * s2 + s3 * s3 + 2.0 * (s4 * s4 + s5 * s5 + s6 * s6));
        }
    }
    __shared__ double red[8], red2[8];
    vn = block_max<8>(vn, red);
    if (snorm) sn = block_max<8>(sn, red2);
    if (threadIdx.x == 0) {
        const int it = *si.step;
        atomic_max_nonneg(&vnorm[it - 1], vn);
        if (snorm) atomic_max_nonneg(&snorm[it - 1], sn);
    }
}

template <typename T>
void pw_launch(const PwDev& pw, const PwFields<T>& F, const StepInfo& s, double* vnorm, double* snorm,
               cudaStream_t st) {
    long long most = 0;
    for (int f = 0; f < pw.nface; ++f) {
        const PwFace& fc = pw.face[f];
        const long long n = (long long)(fc.hi[0] - fc.lo[0] + 1) * (fc.hi[1] - fc.lo[1] + 1) * (fc.hi[2] - fc.lo[2] + 1);
        most = std::max(most, n);
        if (n > 0) pw_inject<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pw, F, f, s);
    }
    if (most > 0) pw_norms<T><<<dim3((unsigned)((most + 255) / 256), pw.nface), 256, 0, st>>>(pw, F, s, vnorm, snorm);
}

}  // namespace

// ------------------------------------------------------- family launchers
template <typename T>
void pw_seismic2(const S2Args<T>& a, const StepInfo& s, cudaStream_t st) {
    PwFields<T> F{};
    F.nx = a.nx; F.ny = 1; F.nz = a.nz;
    F.v[0] = a.f[S2_VX]; F.v[2] = a.f[S2_VZ];
    F.s[0] = a.f[S2_SXX]; F.s[2] = a.f[S2_SZZ]; F.s[4] = a.f[S2_SXZ];
    // C21 slots used by the 2D rows: c11 (0), c13 (2), c15 (4), c33 (11), c35 (13), c55 (18)
    F.C[0] = a.m[S2_C11]; F.C[2] = a.m[S2_C13]; F.C[4] = a.m[S2_C15];
    F.C[11] = a.m[S2_C33]; F.C[13] = a.m[S2_C35]; F.C[18] = a.m[S2_C55];
    pw_launch<T>(a.pw, F, s, a.norms, nullptr, st);
}

template <typename T>
void pw_seismic25(const S25Args<T>& a, const StepInfo& s, cudaStream_t st) {
    PwFields<T> F{};
    F.nx = a.nx; F.ny = 1; F.nz = a.nz; F.cplx = 1; F.stress_tmp = 1;
    for (int d = 0; d < 3; ++d) F.v[d] = a.f[d];
    // S25 field order: vx vy vz sxx sxy sxz syy syz szz
    F.s[0] = a.f[3]; F.s[1] = a.f[6]; F.s[2] = a.f[8]; F.s[3] = a.f[7]; F.s[4] = a.f[5]; F.s[5] = a.f[4];
    for (int q = 0; q < 21; ++q) F.C[q] = a.C[q];
    pw_launch<T>(a.pw, F, s, a.norms, nullptr, st);
}

template <typename T>
void pw_seismic3(const S3Args<T>& a, const StepInfo& s, cudaStream_t st) {
    PwFields<T> F{};
    F.nx = a.nx; F.ny = a.ny; F.nz = a.nz;
    for (int d = 0; d < 3; ++d) F.v[d] = a.f[d];
    // S3 field order: vx vy vz sxx sxy sxz syy syz szz
    F.s[0] = a.f[3]; F.s[1] = a.f[6]; F.s[2] = a.f[8]; F.s[3] = a.f[7]; F.s[4] = a.f[5]; F.s[5] = a.f[4];
    for (int q = 0; q < 21; ++q) F.C[q] = a.C[q];
    pw_launch<T>(a.pw, F, s, a.norms, a.norms + a.nt, st);
}

template <typename T>
void pw_electromag2(const E2Args<T>& a, const StepInfo& s, cudaStream_t st) {
    PwFields<T> F{};
    F.nx = a.nx; F.ny = 1; F.nz = a.nz;
    F.v[0] = a.f[E2_EX]; F.v[2] = a.f[E2_EZ];
    F.h[1] = a.f[E2_HY];
    pw_launch<T>(a.pw, F, s, a.norms, nullptr, st);
}

template <typename T>
void pw_electromag3(const E3Args<T>& a, const StepInfo& s, cudaStream_t st) {
    PwFields<T> F{};
    F.nx = a.nx; F.ny = a.ny; F.nz = a.nz;
    for (int d = 0; d < 3; ++d) { F.v[d] = a.f[d]; F.h[d] = a.f[3 + d]; }
    pw_launch<T>(a.pw, F, s, a.norms, nullptr, st);
}

template void pw_seismic2<float>(const S2Args<float>&, const StepInfo&, cudaStream_t);
template void pw_seismic2<double>(const S2Args<double>&, const StepInfo&, cudaStream_t);
template void pw_seismic25<float>(const S25Args<float>&, const StepInfo&, cudaStream_t);
template void pw_seismic25<double>(const S25Args<double>&, const StepInfo&, cudaStream_t);
template void pw_seismic3<float>(const S3Args<float>&, const StepInfo&, cudaStream_t);
template void pw_seismic3<double>(const S3Args<double>&, const StepInfo&, cudaStream_t);
template void pw_electromag2<float>(const E2Args<float>&, const StepInfo&, cudaStream_t);
template void pw_electromag2<double>(const E2Args<double>&, const StepInfo&, cudaStream_t);
template void pw_electromag3<float>(const E3Args<float>&, const StepInfo&, cudaStream_t);
template void pw_electromag3<double>(const E3Args<double>&, const StepInfo&, cudaStream_t);

// ---------------------------------------------------------- host set-up
// Fill `out` for family/domain/source and the plane-wave parameters; model
// holds the family's host FP64 slots (stiffness and rho, or permittivity).
// Returns 0 or a SEIDART_ERR_* code with `why` set.
int pw_setup(int family, const SeidartDomain* dom, const SeidartSource* src, const SeidartPlaneWave* in,
             const double* const* model, PwDev* out, std::string& why) {
    PwDev pw{};
    const bool em = family == SEIDART_ELECTROMAG2 || family == SEIDART_ELECTROMAG3 || family == SEIDART_ELECTROMAG25;
    const bool three = family == SEIDART_SEISMIC3 || family == SEIDART_ELECTROMAG3;
    if (family == SEIDART_ELECTROMAG25) {
        // the reference sets it up but never injects it (cpmlfdtd.f08:2937-2975, :3261-3266)
        *out = pw;
        return SEIDART_OK;
    }
    if (in->kind == SEIDART_PW_P && em) { why = "a P-wave plane wave is an elastic source"; return SEIDART_ERR_ARG; }
    const int nx = dom->nx, ny = three ? dom->ny : 1, nz = dom->nz, cp = dom->cpml;
    const size_t N = (size_t)nx * ny * nz;
    pw.on = 1;
    pw.em = em ? 1 : 0;
    pw.wavelet = in->wavelet;
    pw.amp = in->amplitude;
    pw.f0 = in->frequency;
    pw.dt = src->dt;
    pw.h[0] = dom->dx; pw.h[1] = three ? dom->dy : 1.0; pw.h[2] = dom->dz;
    if (!(pw.f0 > 0.0)) { why = "plane-wave source_frequency must be positive"; return SEIDART_ERR_ARG; }
    direction(in->x_z_rotation, in->x_y_rotation, in->y_z_rotation, pw.p, pw.ehat);
    if (in->kind == SEIDART_PW_P) for (int d = 0; d < 3; ++d) pw.ehat[d] = pw.p[d];
    // hhat = p x ehat / |p x ehat| (boundary_em_field, plane_wave_source.f08:181-187)
    const double* p = pw.p;
    const double* e = pw.ehat;
    double hh[3] = {p[1] * e[2] - p[2] * e[1], p[2] * e[0] - p[0] * e[2], p[0] * e[1] - p[1] * e[0]};
    const double hn = norm3(hh);
    for (int d = 0; d < 3; ++d) pw.hhat[d] = hn > 0.0 ? hh[d] / hn : hh[d];
    // faces (select_injection_faces, eps 1e-6) and the reference point
    const double eps = 1.0e-6;
    const double lo[3] = {dom->dx * (1 + cp), dom->dy * (1 + cp), dom->dz * (1 + cp)};
    const double hi[3] = {dom->dx * (nx - cp), dom->dy * (dom->ny - cp), dom->dz * (nz - cp)};
    for (int d = 0; d < 3; ++d) pw.loc[d] = 0.5 * (lo[d] + hi[d]);
    bool active[3] = {false, false, false};
    for (int d = 0; d < 3; ++d) {
        if (d == 1 && !three) continue;  // the 2D solvers have no y faces
        if (p[d] > eps) { pw.loc[d] = lo[d]; active[d] = true; }
        if (p[d] < -eps) { pw.loc[d] = hi[d]; active[d] = true; }
    }
    for (int d = 0; d < 3; ++d) pw.r0[d] = pw.loc[d];
    if (!three) pw.r0[1] = 0.0;
    // index ranges of the face loops (1-based in the reference)
    const int inset = family == SEIDART_ELECTROMAG3 ? 3 : 2;  // cpml+3 .. n-cpml-2 for electromag3
    const int n3[3] = {nx, ny, nz};
    int rlo[3], rhi[3];
    for (int d = 0; d < 3; ++d) {
        rlo[d] = cp + inset - 1;              // 0-based
        rhi[d] = n3[d] - cp - (inset - 1) - 1;
    }
    if (!three) { rlo[1] = 0; rhi[1] = 0; }
    pw.nface = 0;
    for (int d = 0; d < 3; ++d) {
        if (!active[d]) continue;
        PwFace f{};
        f.axis = d;
        f.fixed = (int)lround(pw.loc[d] / pw.h[d]) - 1;  // nint(XLOC / dx), 0-based
        if (f.fixed < 0 || f.fixed >= n3[d]) { why = "plane-wave injection face outside the grid"; return SEIDART_ERR_ARG; }
        for (int q = 0; q < 3; ++q) {
            f.lo[q] = q == d ? f.fixed : rlo[q];
            f.hi[q] = q == d ? f.fixed : rhi[q];
        }
        pw.face[pw.nface++] = f;
    }
    // background speed
    if (em) {
        const bool two = family == SEIDART_ELECTROMAG2;
        double eps_min;
        if (two) {
            const double* g[3] = {model[E2_E11], model[E2_E13], model[E2_E33]};
            // eigen2(e11, e13, 0, e33, 0, 0): lambda(2:3) of diag-block + zero (array_eigenvalues2_2)
            eps_min = over_tuples(N, 3, g, INFINITY,
                                  [](const double* t) {
                                      double a[9] = {t[0], t[1], 0, t[1], t[2], 0, 0, 0, 0}, l[3];
                                      jacobi_eigenvalues(3, a, l);
                                      return l[1];
                                  },
                                  [](double x, double y) { return y < x ? y : x; });
        } else {
            const double* g[6] = {model[E3_E11], model[E3_E12], model[E3_E13], model[E3_E22], model[E3_E23], model[E3_E33]};
            eps_min = over_tuples(N, 6, g, INFINITY,
                                  [](const double* t) {
                                      double a[9] = {t[0], t[1], t[2], t[1], t[3], t[4], t[2], t[4], t[5]}, l[3];
                                      jacobi_eigenvalues(3, a, l);
                                      return l[0];
                                  },
                                  [](double x, double y) { return y < x ? y : x; });
        }
        const double c0 = 2.99792458e8, mu0 = 4.0 * kPi * 1.0e-7, eps0 = 8.85418782e-12;  // constants.f08
        pw.v = c0 / sqrt(eps_min);
        pw.eta = sqrt(mu0 / (eps0 * eps_min));
    } else {
        double cmax;
        const double* rho;
        if (family == SEIDART_SEISMIC2) {
            const double* g[6] = {model[S2_C11], model[S2_C13], model[S2_C15], model[S2_C33], model[S2_C35], model[S2_C55]};
            cmax = over_tuples(N, 6, g, -INFINITY,
                               [](const double* t) {
                                   double c21[21] = {0};
                                   c21[0] = t[0]; c21[2] = t[1]; c21[4] = t[2];
                                   c21[11] = t[3]; c21[13] = t[4]; c21[18] = t[5];
                                   return mandel_max_eig(c21);
                               },
                               [](double x, double y) { return y > x ? y : x; });
            rho = model[S2_RHO];
        } else {
            const double* g[21];
            for (int q = 0; q < 21; ++q) g[q] = model[q];
            cmax = over_tuples(N, 21, g, -INFINITY, [](const double* t) { return mandel_max_eig(t); },
                               [](double x, double y) { return y > x ? y : x; });
            rho = model[SEIDART_RHO3];
        }
        double rmin = INFINITY;
        for (size_t c = 0; c < N; ++c) rmin = std::min(rmin, rho[c]);
        pw.v = sqrt(cmax / rmin);
    }
    if (!(pw.v > 0.0) || !isfinite(pw.v)) { why = "plane-wave background speed is not positive"; return SEIDART_ERR_ARG; }
    *out = pw;
    return SEIDART_OK;
}

extern "C" {
// Host-side set-up figures of a plane-wave source, for callers and tests:
// out[0] background speed, out[1] impedance (EM; 0 elastic), out[2..4] the
// propagation direction p, out[5..7] the polarisation ehat, out[8] the
// number of injection faces, out[9..11] their axes (0 x, 1 y, 2 z; -1 unused)
// and out[12..14] their fixed 0-based indices.
int seidart_plane_wave_setup(int family, const SeidartDomain* dom, const SeidartSource* src,
                             const SeidartPlaneWave* pw, const double* const* model, double* out) {
    if (!dom || !src || !pw || !model || !out) return SEIDART_ERR_ARG;
    PwDev d{};
    std::string why;
    const int rc = pw_setup(family, dom, src, pw, model, &d, why);
    if (rc != SEIDART_OK) return rc;
    out[0] = d.v;
    out[1] = d.eta;
    for (int q = 0; q < 3; ++q) { out[2 + q] = d.p[q]; out[5 + q] = d.ehat[q]; }
    out[8] = d.nface;
    for (int f = 0; f < 3; ++f) {
        out[9 + f] = f < d.nface ? d.face[f].axis : -1;
        out[12 + f] = f < d.nface ? d.face[f].fixed : -1;
    }
    return SEIDART_OK;
}
}  // extern "C"
