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
        rc = fn(*head, *common)
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
