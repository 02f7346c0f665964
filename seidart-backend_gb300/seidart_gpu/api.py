"""numpy-level interface to the GPU solvers.

A :class:`Problem` holds one model exactly as the reference solvers consume
it: padded grids in Fortran order (x fastest; complex128 for 2.5D), source
time series, initial fields and receiver cells.  :class:`Solver` owns the
device copy of a Problem (through the C ABI) and advances it; :func:`run`
mirrors one call of a reference subroutine (``seismic2(domain, source, ...)``
in src/fortran/cpmlfdtd.f08) without its per-step file output.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (ELECTROMAG2, ELECTROMAG3, ELECTROMAG25, FP32, FP64, SEISMIC2, SEISMIC3, SEISMIC25, Domain, Source, check,
                   lib, ptr_array)

FAMILY_NAMES = {SEISMIC2: "seismic2", SEISMIC25: "seismic25", SEISMIC3: "seismic3",
                ELECTROMAG2: "electromag2", ELECTROMAG25: "electromag25", ELECTROMAG3: "electromag3"}
DENSITY_CODES = {"harmonic": 1, "geometric": 2, "arithmetic": 3, "none": 4}

# Slot names in C-ABI order (include/seidart_gpu.h)
C21 = ["c11", "c12", "c13", "c14", "c15", "c16", "c22", "c23", "c24", "c25", "c26",
       "c33", "c34", "c35", "c36", "c44", "c45", "c46", "c55", "c56", "c66"]
CPML6 = ["kappa", "kappa_half", "acoef", "acoef_half", "bcoef", "bcoef_half"]
MODEL_SLOTS = {
    SEISMIC2: ["c11", "c13", "c15", "c33", "c35", "c55", "rho", "gamma_x", "gamma_z", "gamma_xz", *CPML6],
    SEISMIC25: [*C21, "rho", "gamma_x", "gamma_y", "gamma_z", "gamma_xy", "gamma_yz", "gamma_xz", *CPML6],
    SEISMIC3: [*C21, "rho", "gamma_x", "gamma_y", "gamma_z", "gamma_xy", "gamma_yz", "gamma_xz", *CPML6],
    ELECTROMAG2: ["e11", "e13", "e33", "s11", "s13", "s33", *CPML6],
    ELECTROMAG25: ["e11", "e12", "e13", "e22", "e23", "e33", "s11", "s12", "s13", "s22", "s23", "s33", *CPML6],
    ELECTROMAG3: ["e11", "e12", "e13", "e22", "e23", "e33", "s11", "s12", "s13", "s22", "s23", "s33", *CPML6],
}
SRC_SLOTS = {
    SEISMIC2: ["x", "z", "xx", "xz", "zz"],
    SEISMIC25: ["x", "y", "z", "xx", "xy", "xz", "yy", "yz", "zz"],
    SEISMIC3: ["x", "y", "z", "xx", "xy", "xz", "yy", "yz", "zz"],
    ELECTROMAG2: ["x", "z"],
    ELECTROMAG25: ["x", "y", "z"],
    ELECTROMAG3: ["x", "y", "z"],
}
FIELD_SLOTS = {
    SEISMIC2: ["vx", "vz", "sigmaxx", "sigmazz", "sigmaxz"],
    SEISMIC25: ["vx", "vy", "vz", "sigmaxx", "sigmaxy", "sigmaxz", "sigmayy", "sigmayz", "sigmazz"],
    SEISMIC3: ["vx", "vy", "vz", "sigmaxx", "sigmaxy", "sigmaxz", "sigmayy", "sigmayz", "sigmazz"],
    ELECTROMAG2: ["Ex", "Ez", "Hy"],
    ELECTROMAG25: ["Ex", "Ey", "Ez", "Hx", "Hy", "Hz"],
    ELECTROMAG3: ["Ex", "Ey", "Ez", "Hx", "Hy", "Hz"],
}


def layout(family: int) -> dict:
    vals = [C.c_int() for _ in range(6)]
    check(lib().seidart_layout(family, *[C.byref(v) for v in vals]))
    keys = ["nmodel", "nsrc", "nfield", "nmem", "is_complex", "nrec_comp"]
    return {k: v.value for k, v in zip(keys, vals)}


@dataclass
class Problem:
    """One model + source + receivers, in the reference's array layout."""
    family: int
    nx: int
    nz: int
    dx: float
    dz: float
    dt: float
    time_steps: int
    cpml: int
    xind: int            # interior source indices (cell = ind + cpml, 1-based)
    zind: int
    model: dict          # slot name -> float64 grid (Fortran order, padded)
    src: dict = field(default_factory=dict)      # slot name -> float64[time_steps]
    fields0: dict = field(default_factory=dict)  # slot name -> initial grid
    receivers: np.ndarray | None = None          # 0-based linear cell indices
    ny: int = 1
    dy: float = 1.0
    yind: int = 0
    ky: float = 0.0
    density: str = "arithmetic"
    meta: dict = field(default_factory=dict)
    # plane-wave source: {"kind": "pw" | "pwp", "wavelet": "gaus0|1|2",
    # "x_z_rotation", "x_y_rotation", "y_z_rotation" (degrees), "amplitude",
    # "frequency"}; None = point sources from `src`
    plane_wave: dict | None = None

    def plane_wave_struct(self):
        """The plane_wave dict as a SeidartPlaneWave (None without one)."""
        pw = self.plane_wave
        if not pw:
            return None
        kind = pw.get("kind", "pw")
        return _lib.PlaneWave(_lib.PW_P if kind in ("pwp", "pw_p", "pw-p") else _lib.PW_S,
                              _lib.WAVELETS.get(pw.get("wavelet", "gaus0"), 0),
                              float(pw.get("x_z_rotation", 0.0)), float(pw.get("x_y_rotation", 0.0)),
                              float(pw.get("y_z_rotation", 0.0)), float(pw.get("amplitude", 1.0)),
                              float(pw["frequency"]))

    @property
    def shape(self) -> tuple:
        return (self.nx, self.ny, self.nz) if self.is3d else (self.nx, self.nz)

    @property
    def is3d(self) -> bool:
        return self.family in (SEISMIC3, ELECTROMAG3)

    @property
    def ncell(self) -> int:
        return int(np.prod(self.shape))

    @property
    def is_complex(self) -> bool:
        return self.family in (SEISMIC25, ELECTROMAG25)

    def domain(self) -> Domain:
        dim = 3.0 if self.is3d else (2.5 if self.is_complex else 2.0)
        return Domain(dim, self.nx, self.ny, self.nz, self.dx, self.dy, self.dz, self.cpml)

    def source(self) -> Source:
        return Source(self.dt, self.time_steps, self.xind, self.yind, self.zind, self.ky)

    def density_code(self) -> int:
        return DENSITY_CODES[self.density]

    def model_list(self) -> list:
        out = []
        for name in MODEL_SLOTS[self.family]:
            a = np.asfortranarray(self.model[name], dtype=np.float64)
            if a.shape != self.shape:
                raise ValueError(f"model array {name} has shape {a.shape}, expected {self.shape}")
            out.append(a)
        return out

    def src_list(self) -> list:
        out = []
        for name in SRC_SLOTS[self.family]:
            s = self.src.get(name)
            if s is not None:
                s = np.ascontiguousarray(s, dtype=np.float64)
                if s.shape != (self.time_steps,):
                    raise ValueError(f"source series {name} must have {self.time_steps} samples")
            out.append(s)
        return out

    def field_list(self) -> list:
        dt = np.complex128 if self.is_complex else np.float64
        out = []
        for name in FIELD_SLOTS[self.family]:
            f = self.fields0.get(name)
            out.append(np.zeros(self.shape, dtype=dt, order="F") if f is None
                       else np.asfortranarray(f, dtype=dt).copy(order="F"))
        return out

    def given_fields(self) -> list:
        """Initial fields the problem sets, None for the ones it leaves at zero."""
        dt = np.complex128 if self.is_complex else np.float64
        out = []
        for name in FIELD_SLOTS[self.family]:
            f = self.fields0.get(name)
            if f is not None:
                f = np.asfortranarray(f, dtype=dt)
                if f.shape != self.shape:
                    raise ValueError(f"initial field {name} has shape {f.shape}, expected {self.shape}")
            out.append(f)
        return out

    def receiver_array(self) -> np.ndarray:
        if self.receivers is None:
            return np.zeros(0, dtype=np.int32)
        return np.ascontiguousarray(self.receivers, dtype=np.int32)

    def source_cell(self) -> int:
        """0-based linear index of the source cell (ind + cpml, 1-based)."""
        i, j, k = self.xind + self.cpml - 1, self.yind + self.cpml - 1, self.zind + self.cpml - 1
        if self.is3d:
            return i + self.nx * (j + self.ny * k)
        return i + self.nx * k


def _is_device_grid(a) -> bool:
    return hasattr(a, "data_ptr") and bool(getattr(a, "is_cuda", False))


class _DevicePtr:
    """A CUDA tensor standing in a model slot: ptr_array passes its address."""

    def __init__(self, t, ncell: int, name: str):
        import torch
        if t.dtype != torch.float64 or t.numel() != ncell or not t.is_contiguous():
            raise ValueError(f"device model grid {name} must be a contiguous float64 CUDA tensor of {ncell} cells "
                             "(row-major (nz, nx) / (nz, ny, nx), the Fortran layout)")
        self.t = t
        self.ctypes = type("_P", (), {"data": t.data_ptr()})()


def _model_arrays(problem: Problem) -> list:
    """The model slots for seidart_solver_create: host FP64 grids, or for
    seismic2 / seismic3 CUDA FP64 tensors (the device material pre-pass's
    output) in the stiffness, density and attenuation slots."""
    names = MODEL_SLOTS[problem.family]
    if not any(_is_device_grid(problem.model[n]) for n in names):
        return problem.model_list()
    if problem.plane_wave:
        raise ValueError("plane-wave set-up reads the stiffness on the host: pass host model grids")
    out = []
    for n in names:
        a = problem.model[n]
        if _is_device_grid(a):
            out.append(_DevicePtr(a, problem.ncell, n))
        else:
            a = np.asfortranarray(a, dtype=np.float64)
            if a.shape != problem.shape:
                raise ValueError(f"model array {n} has shape {a.shape}, expected {problem.shape}")
            out.append(a)
    return out


class Solver:
    """Device copy of a Problem, advanced on the GPU."""

    def __init__(self, problem: Problem, precision: int = FP64):
        self.problem = problem
        self.precision = precision
        self.lay = layout(problem.family)
        self._model = _model_arrays(problem)    # keep alive during create
        self._src = problem.src_list()
        rec = problem.receiver_array()
        self._rec = rec
        h = C.c_void_p()
        check(lib().seidart_solver_create(C.byref(h), problem.family, precision, C.byref(problem.domain()),
                                          C.byref(problem.source()), problem.density_code(),
                                          ptr_array(self._model), ptr_array(self._src), len(rec),
                                          rec.ctypes.data if len(rec) else None))
        self.handle = h
        # the device state starts at zero: only the initial fields the problem sets travel
        self.set_fields(problem.given_fields())
        pw = problem.plane_wave_struct()
        if pw is not None:
            check(lib().seidart_solver_set_plane_wave(self.handle, C.byref(pw), ptr_array(self._model)))

    # ------------------------------------------------------------------ state
    def set_fields(self, fields: list) -> None:
        arrs = [None if f is None else np.asfortranarray(f) for f in fields]
        check(lib().seidart_solver_set_fields(self.handle, ptr_array(arrs)))

    def get_fields(self) -> list:
        out = self.problem.field_list()
        check(lib().seidart_solver_get_fields(self.handle, ptr_array(out)))
        return out

    def get_memory(self) -> list:
        dt = np.complex128 if self.problem.is_complex else np.float64
        out = [np.zeros(self.problem.shape, dtype=dt, order="F") for _ in range(self.lay["nmem"])]
        check(lib().seidart_solver_get_memory(self.handle, ptr_array(out)))
        return out

    # ------------------------------------------------------------------ steps
    def step(self, n: int) -> None:
        check(lib().seidart_solver_step(self.handle, int(n)))

    def profile(self, n: int) -> dict:
        """Advance ``n`` steps kernel by kernel with CUDA events between launches.
        Returns total ms and, per kernel name, summed ms and launch count."""
        tot = C.c_double()
        km = (C.c_double * 8)()
        kl = (C.c_int * 8)()
        names = C.create_string_buffer(8 * 48)
        check(lib().seidart_solver_profile(self.handle, int(n), C.byref(tot), km, kl, names, 48))
        out = {"total_ms": tot.value, "kernels": {}}
        for k in range(8):
            if kl[k]:
                nm = names.raw[k * 48:(k + 1) * 48].split(b"\0")[0].decode()
                out["kernels"][nm] = {"ms": km[k], "launches": kl[k]}
        return out

    def sync(self) -> None:
        check(lib().seidart_solver_sync(self.handle))

    @property
    def steps_done(self) -> int:
        return lib().seidart_solver_steps_done(self.handle)

    def material_count(self) -> int:
        """Materials of the FP32 3D material-indexed coefficient layout (0:
        the per-cell arrays are used)."""
        return lib().seidart_solver_material_count(self.handle)

    def stress_memory_arrays(self) -> int:
        """Stress-loop C-PML memory arrays a seismic3 solver advances (21
        merged or 36); get_memory returns the 36 either way."""
        return lib().seidart_solver_stress_memory_arrays(self.handle)

    def cpml_tuples(self) -> int:
        """Tuples of the FP32 3D indexed C-PML coefficients (0: the grids)."""
        return lib().seidart_solver_cpml_tuples(self.handle)

    @property
    def launches(self) -> int:
        return lib().seidart_solver_launches(self.handle)

    def set_wait(self, limit: int, probe_bytes: int = 0) -> None:
        """Bound (in polls) of the FP32 3D kernels' device waits; probe_bytes > 0
        is the test hook that makes one CTA's waits run out (see
        seidart_solver_set_wait in include/seidart_gpu.h)."""
        check(lib().seidart_solver_set_wait(self.handle, int(limit), int(probe_bytes)))

    def field_ptr(self, slot: int) -> int:
        return lib().seidart_solver_field_ptr(self.handle, slot)

    def set_stream(self, stream_ptr: int | None) -> None:
        check(lib().seidart_solver_set_stream(self.handle, stream_ptr))

    def traces(self):
        """(traces [steps][ncomp][nrec] (complex for 2.5D), norms [steps] or [2][steps])."""
        n = self.steps_done
        nrec = len(self._rec)
        ncomp = self.lay["nrec_comp"]
        dt = np.complex128 if self.problem.is_complex else np.float64
        tr = np.zeros((n, ncomp, nrec), dtype=dt)
        nn = 2 if self.problem.family == SEISMIC3 else 1
        nrm = np.zeros((nn, n))
        check(lib().seidart_solver_traces(self.handle, tr.ctypes.data if nrec else None, nrm.ctypes.data))
        return tr, (nrm if nn == 2 else nrm[0])

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().seidart_solver_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run(problem: Problem, precision: int = FP64, nsteps: int | None = None) -> dict:
    """Run ``nsteps`` (default: all) steps; returns fields, memory, traces, norms."""
    with Solver(problem, precision) as s:
        s.step(problem.time_steps if nsteps is None else nsteps)
        s.sync()
        tr, nrm = s.traces()
        return {"fields": s.get_fields(), "memory": s.get_memory(), "traces": tr, "norms": nrm}
