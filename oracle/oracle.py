"""ctypes loader for the CPU restatement of the reference time loops.

TEST INFRASTRUCTURE ONLY: the checker for the GPU solvers (tests, the smoke
check and the CPU-baseline leg of the benchmark).  Parity status: UNPINNED --
the reference ships no golden vectors and cannot be compiled here.

``run_oracle(problem, nsteps)`` advances a ``seidart_gpu.api.Problem`` on the
CPU and returns the same dict as ``seidart_gpu.api.run``: fields, full-grid
CPML memory arrays, receiver traces and max-norm series.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
NAMES = {1: "oracle_seismic2", 2: "oracle_seismic25", 3: "oracle_seismic3", 4: "oracle_electromag2",
         5: "oracle_electromag25", 6: "oracle_electromag3"}
NMEM = {1: 12, 2: 30, 3: 45, 4: 4, 5: 8, 6: 12}
NCOMP = {1: 2, 2: 3, 3: 3, 4: 2, 5: 3, 6: 3}
_libs = {}

EPS0 = 8.85418782e-12                       # constants.f08
MU0 = 4.0 * 3.141592653589793238462643 * 1.0e-7
CLIGHT = 2.99792458e8


class OraclePw(C.Structure):
    _fields_ = [("on", C.c_int), ("p_wave", C.c_int), ("wavelet", C.c_int), ("x_z_rotation", C.c_double),
                ("x_y_rotation", C.c_double), ("y_z_rotation", C.c_double), ("amplitude", C.c_double),
                ("frequency", C.c_double), ("v", C.c_double), ("eta", C.c_double)]


def _unique_rows(arrs):
    m = np.stack([np.asarray(a, dtype=np.float64).ravel(order="F") for a in arrs], axis=1)
    return np.unique(m, axis=0)


def plane_wave_background(problem) -> tuple:
    """(v, eta) of a plane-wave run as the reference computes them with LAPACK
    (tensor_operations.f08, array_eigenvalues*): elastic v = sqrt(max
    eigenvalue of the Mandel stiffness / min rho); EM v = c / sqrt(eps_min),
    eta = sqrt(mu0 / (eps0 eps_min)).  numpy's eigvalsh is LAPACK as well."""
    m = problem.model
    fam = problem.family
    if fam in (1, 2, 3):
        if fam == 1:
            names = ("c11", "c13", "c15", "c33", "c35", "c55")
            rows = _unique_rows([m[k] for k in names])
            A = np.zeros((len(rows), 6, 6))
            for q, (a, b) in enumerate(((0, 0), (0, 2), (0, 4), (2, 2), (2, 4), (4, 4))):
                A[:, a, b] = A[:, b, a] = rows[:, q]
        else:
            c21 = [f"c{i}{j}" for i in range(1, 7) for j in range(i, 7)]
            rows = _unique_rows([m[k] for k in c21])
            A = np.zeros((len(rows), 6, 6))
            q = 0
            for a in range(6):
                for b in range(a, 6):
                    A[:, a, b] = A[:, b, a] = rows[:, q]
                    q += 1
        s = np.array([1.0, 1.0, 1.0, np.sqrt(2.0), np.sqrt(2.0), np.sqrt(2.0)])
        A = A * s[None, :, None] * s[None, None, :]
        lam = np.linalg.eigvalsh(A)
        return float(np.sqrt(lam.max() / np.min(m["rho"]))), 0.0
    if fam == 4:
        rows = _unique_rows([m["e11"], m["e13"], m["e33"]])
        A = np.zeros((len(rows), 3, 3))
        A[:, 0, 0], A[:, 0, 1], A[:, 1, 0], A[:, 1, 1] = rows[:, 0], rows[:, 1], rows[:, 1], rows[:, 2]
        eps_min = float(np.linalg.eigvalsh(A)[:, 1].min())   # lambda(2:3) of eigen2
    else:
        rows = _unique_rows([m[k] for k in ("e11", "e12", "e13", "e22", "e23", "e33")])
        A = np.zeros((len(rows), 3, 3))
        for q, (a, b) in enumerate(((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))):
            A[:, a, b] = A[:, b, a] = rows[:, q]
        eps_min = float(np.linalg.eigvalsh(A).min())
    return CLIGHT / np.sqrt(eps_min), float(np.sqrt(MU0 / (EPS0 * eps_min)))


def oracle_plane_wave(problem):
    """OraclePw for a Problem with a plane_wave dict (None without one)."""
    pw = problem.plane_wave
    if not pw:
        return None
    v, eta = plane_wave_background(problem)
    kind = pw.get("kind", "pw")
    return OraclePw(1, 1 if kind in ("pwp", "pw_p", "pw-p") else 0,
                    {"gaus1": 1, "gaus2": 2}.get(pw.get("wavelet", "gaus0"), 0),
                    float(pw.get("x_z_rotation", 0.0)), float(pw.get("x_y_rotation", 0.0)),
                    float(pw.get("y_z_rotation", 0.0)), float(pw.get("amplitude", 1.0)), float(pw["frequency"]),
                    v, eta)


def build() -> None:
    """Compile both oracle builds (parity and OpenMP baseline) with make."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def load(kind: str = "parity") -> C.CDLL:
    """kind = 'parity' (no fast-math, no FMA contraction) or 'omp' (the
    reference's production flags, OpenMP)."""
    if kind not in _libs:
        path = BUILD / ("liboracle.so" if kind == "parity" else "liboracle_omp.so")
        if not path.exists():
            build()
        L = C.CDLL(str(path))
        vp = C.c_void_p
        for fam, name in NAMES.items():
            fn = getattr(L, name)
            fn.restype = C.c_int
            # (domain, source, [density], model, src, fields, mem, it0, nsteps, nrec, rec, traces, norms)
            head = [vp, vp, C.c_int] if fam in (1, 2, 3) else [vp, vp]
            fn.argtypes = head + [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.oracle_threads.restype = C.c_int
        L.oracle_set_plane_wave.restype = None
        L.oracle_set_plane_wave.argtypes = [C.c_void_p]
        _libs[kind] = L
    return _libs[kind]


def _ptrs(arrs):
    out = (C.c_void_p * max(len(arrs), 1))()
    for q, a in enumerate(arrs):
        out[q] = None if a is None else a.ctypes.data
    return out


class OracleState:
    """Fields + full-grid CPML memories of one problem on the CPU."""

    def __init__(self, problem, kind: str = "parity"):
        self.p = problem
        self.lib = load(kind)
        self.model = problem.model_list()
        self.src = problem.src_list()
        self.fields = problem.field_list()
        dt = np.complex128 if problem.is_complex else np.float64
        self.mem = [np.zeros(problem.shape, dtype=dt, order="F") for _ in range(NMEM[problem.family])]
        self.rec = problem.receiver_array()
        self.steps_done = 0
        self.traces = []
        self.norms = []
        self.pw = oracle_plane_wave(problem)

    def step(self, n: int) -> int:
        p = self.p
        fam = p.family
        nrec = len(self.rec)
        dt = np.complex128 if p.is_complex else np.float64
        tr = np.zeros((n, NCOMP[fam], nrec), dtype=dt)
        nn = 2 if fam == 3 else 1
        nrm = np.zeros((nn, n))
        fn = getattr(self.lib, NAMES[fam])
        dom, srcd = p.domain(), p.source()
        keep = [_ptrs(self.model), _ptrs(self.src), _ptrs(self.fields), _ptrs(self.mem)]
        common = [C.cast(k, C.c_void_p) for k in keep] + [
            self.steps_done, n, nrec, self.rec.ctypes.data if nrec else None,
            tr.ctypes.data if nrec else None, nrm.ctypes.data]
        head = [C.addressof(dom), C.addressof(srcd)]
        if fam in (1, 2, 3):
            head.append(p.density_code())
        self.lib.oracle_set_plane_wave(C.addressof(self.pw) if self.pw is not None else None)
        try:
            rc = fn(*head, *common)
        finally:
            self.lib.oracle_set_plane_wave(None)
        if rc < 0:
            raise MemoryError("oracle allocation failed")
        done = n if rc == 0 else rc - self.steps_done
        self.steps_done += done
        self.traces.append(tr[:done])
        self.norms.append(nrm[:, :done])
        return rc

    def result(self) -> dict:
        nrm = np.concatenate(self.norms, axis=1) if self.norms else np.zeros((1, 0))
        return {"fields": self.fields, "memory": self.mem,
                "traces": np.concatenate(self.traces, axis=0) if self.traces else None,
                "norms": nrm if self.p.family == 3 else nrm[0], "blowup": None}


def run_oracle(problem, nsteps: int | None = None, kind: str = "parity") -> dict:
    st = OracleState(problem, kind)
    rc = st.step(problem.time_steps if nsteps is None else nsteps)
    out = st.result()
    out["blowup"] = rc if rc > 0 else None
    return out
