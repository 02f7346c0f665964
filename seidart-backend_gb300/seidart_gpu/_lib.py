"""ctypes binding of libseidart_gpu.so (the C ABI in include/seidart_gpu.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly when the shared object is missing.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libseidart_gpu.so"

SEIDART_OK = 0
ERRORS = {
    -1: "SEIDART_ERR_ARG",
    -2: "SEIDART_ERR_CUDA",
    -3: "SEIDART_ERR_UNSTABLE",
    -4: "SEIDART_ERR_IO",
    -5: "SEIDART_ERR_NOMEM",
    -6: "SEIDART_ERR_TIMEOUT",
    -7: "SEIDART_ERR_UNSUPPORTED",
}

SEISMIC2, SEISMIC25, SEISMIC3, ELECTROMAG2, ELECTROMAG25, ELECTROMAG3 = 1, 2, 3, 4, 5, 6
FP64, FP32, FP64_FAST = 0, 1, 2


class SeidartError(RuntimeError):
    """Error returned by the C ABI; ``code`` is the SEIDART_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class UnstableError(SeidartError):
    """The max-norm exceeded 1e25 (the reference stops with 'code became unstable')."""


class Domain(C.Structure):
    _fields_ = [("dim", C.c_double), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("cpml", C.c_int)]


class Source(C.Structure):
    _fields_ = [("dt", C.c_double), ("time_steps", C.c_int), ("xind", C.c_int), ("yind", C.c_int),
                ("zind", C.c_int), ("ky", C.c_double)]


class PlaneWave(C.Structure):
    """SeidartPlaneWave: kind 1 = transverse ("pw"), 2 = P wave ("pwp");
    wavelet 0 gaus0, 1 gaus1, 2 gaus2; rotations in degrees."""
    _fields_ = [("kind", C.c_int), ("wavelet", C.c_int), ("x_z_rotation", C.c_double),
                ("x_y_rotation", C.c_double), ("y_z_rotation", C.c_double), ("amplitude", C.c_double),
                ("frequency", C.c_double)]


PW_S, PW_P = 1, 2
WAVELETS = {"gaus0": 0, "gaus1": 1, "gaus2": 2}

DPP = C.POINTER(C.c_void_p)

_SIGS = {
    "seidart_layout": (C.c_int, [C.c_int] + [C.POINTER(C.c_int)] * 6),
    "seidart_run": (C.c_int, [C.c_int, C.c_int, C.POINTER(Domain), C.POINTER(Source), C.c_int, DPP, DPP, DPP,
                              C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "seidart_solver_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(Domain),
                                        C.POINTER(Source), C.c_int, DPP, DPP, C.c_int, C.c_void_p]),
    "seidart_solver_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "seidart_solver_set_fields": (C.c_int, [C.c_void_p, DPP]),
    "seidart_solver_set_plane_wave": (C.c_int, [C.c_void_p, C.POINTER(PlaneWave), DPP]),
    "seidart_solver_get_fields": (C.c_int, [C.c_void_p, DPP]),
    "seidart_solver_get_memory": (C.c_int, [C.c_void_p, DPP]),
    "seidart_solver_step": (C.c_int, [C.c_void_p, C.c_int]),
    "seidart_solver_sync": (C.c_int, [C.c_void_p]),
    "seidart_solver_traces": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "seidart_solver_steps_done": (C.c_int, [C.c_void_p]),
    "seidart_solver_material_count": (C.c_int, [C.c_void_p]),
    "seidart_solver_stress_memory_arrays": (C.c_int, [C.c_void_p]),
    "seidart_solver_cpml_tuples": (C.c_int, [C.c_void_p]),
    "seidart_solver_profile": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_int]),
    "seidart_solver_field_ptr": (C.c_void_p, [C.c_void_p, C.c_int]),
    "seidart_solver_launches": (C.c_longlong, [C.c_void_p]),
    "seidart_solver_set_wait": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "seidart_solver_destroy": (C.c_int, [C.c_void_p]),
    "seidart_last_error": (C.c_char_p, []),
}

_lib = None


def lib() -> C.CDLL:
    """Load libseidart_gpu.so (once) and declare the C signatures."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the solvers have no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != SEIDART_OK:
        msg = lib().seidart_last_error().decode(errors="replace")
        if rc == -3:
            raise UnstableError(rc, msg)
        raise SeidartError(rc, msg)


def ptr_array(arrays) -> C.Array:
    """Array of void* from a list of numpy arrays / None (None -> NULL)."""
    out = (C.c_void_p * max(len(arrays), 1))()
    for q, a in enumerate(arrays):
        out[q] = None if a is None else a.ctypes.data
    return out
