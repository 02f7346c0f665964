"""Ragged batches of 2D elastic models in one persistent GPU launch.

``Batch(problems)`` takes seismic2 :class:`~seidart_gpu.api.Problem` objects of
any (uneven) grid sizes sharing one number of time steps; every step of all
models runs inside one cooperative persistent kernel (csrc/batch.cu), FP32
fields.  The tile shape and CTAs per SM are chosen by timing every candidate
on the batch itself (``autotune=True``), after which the models are reset and
their initial fields loaded.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SEISMIC2, Domain, SeidartError, Source, UnstableError, lib, ptr_array
from .api import Problem

_DECL = False


def _declare():
    global _DECL
    if _DECL:
        return
    L = lib()
    vp, i, ll = C.c_void_p, C.c_int, C.c_longlong
    sig = {
        "seidart_batch_create": (i, [C.POINTER(vp), i, vp, vp, vp, vp, vp, vp, vp]),
        "seidart_batch_autotune": (i, [vp, i, C.POINTER(i), C.POINTER(i)]),
        "seidart_batch_tuning": (i, [vp, i, C.POINTER(i), C.POINTER(i), vp, vp]),
        "seidart_batch_set_config": (i, [vp, i, i]),
        "seidart_batch_step": (i, [vp, i, i]),
        "seidart_batch_sync": (i, [vp]),
        "seidart_batch_force_timeout": (i, [vp, ll]),
        "seidart_batch_model": (vp, [vp, i]),
        "seidart_batch_steps_done": (i, [vp]),
        "seidart_batch_launches": (ll, [vp]),
        "seidart_batch_graph_launches": (ll, [vp]),
        "seidart_batch_config": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
        "seidart_batch_num_variants": (i, []),
        "seidart_batch_variant_walk": (C.c_char_p, [i]),
        "seidart_batch_material_count": (i, [vp, i]),
        "seidart_batch_destroy": (i, [vp]),
        "seidart_batch_last_error": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    _DECL = True


def _check(rc):
    if rc != 0:
        msg = lib().seidart_batch_last_error().decode(errors="replace")
        if rc == -3:
            raise UnstableError(rc, msg)
        raise SeidartError(rc, msg)


class Batch:
    def __init__(self, problems: list[Problem], autotune: bool = True, trial_steps: int = 24):
        _declare()
        L = lib()
        if not problems or any(p.family != SEISMIC2 for p in problems):
            raise ValueError("a Batch holds seismic2 problems")
        self.problems = problems
        n = len(problems)
        self._keep = []
        doms = (Domain * n)(*[p.domain() for p in problems])
        srcs = (Source * n)(*[p.source() for p in problems])
        dens = (C.c_int * n)(*[p.density_code() for p in problems])
        mptrs = (C.c_void_p * n)()
        sptrs = (C.c_void_p * n)()
        rptrs = (C.c_void_p * n)()
        nrec = (C.c_int * n)()
        for m, p in enumerate(problems):
            ml, sl, rec = p.model_list(), p.src_list(), p.receiver_array()
            ma, sa = ptr_array(ml), ptr_array(sl)
            self._keep += [ml, sl, rec, ma, sa]
            mptrs[m] = C.cast(ma, C.c_void_p)
            sptrs[m] = C.cast(sa, C.c_void_p)
            rptrs[m] = rec.ctypes.data if len(rec) else None
            nrec[m] = len(rec)
        h = C.c_void_p()
        _check(L.seidart_batch_create(C.byref(h), n, C.addressof(doms), C.addressof(srcs), C.addressof(dens),
                                      C.addressof(mptrs), C.addressof(sptrs), C.addressof(nrec), C.addressof(rptrs)))
        self.handle = h
        self.tuning = None
        self.variant = 1  # the library's default until autotuned or set
        if autotune:
            v, b = C.c_int(), C.c_int()
            _check(L.seidart_batch_autotune(self.handle, min(trial_steps, problems[0].time_steps),
                                            C.byref(v), C.byref(b)))
            self.variant = v.value
            self.tuning = self._tuning_table()
        for m, p in enumerate(problems):
            self._set_fields(m, p.field_list())

    def _tuning_table(self):
        L = lib()
        out = []
        for v in range(L.seidart_batch_num_variants()):
            tx, ty = C.c_int(), C.c_int()
            bps = (C.c_int * 2)()
            ms = (C.c_double * 2)()
            _check(L.seidart_batch_tuning(self.handle, v, C.byref(tx), C.byref(ty), C.addressof(bps), C.addressof(ms)))
            walk = L.seidart_batch_variant_walk(v).decode()
            for q in range(2):
                if ms[q] >= 0:
                    out.append({"variant": v, "walk": walk, "tile": [tx.value, ty.value], "ctas_per_sm": bps[q],
                                "ms": ms[q]})
        return out

    def config(self) -> dict:
        tx, ty, bps, grid = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib().seidart_batch_config(self.handle, C.byref(tx), C.byref(ty), C.byref(bps), C.byref(grid)))
        return {"variant": self.variant, "walk": lib().seidart_batch_variant_walk(self.variant).decode(),
                "tile": [tx.value, ty.value], "ctas_per_sm": bps.value, "grid": grid.value}

    def set_config(self, variant: int, ctas_per_sm: int) -> None:
        """Use kernel variant ``variant`` (0 .. num_variants-1) with the given
        CTAs per SM instead of the autotuned choice."""
        _check(lib().seidart_batch_set_config(self.handle, int(variant), int(ctas_per_sm)))
        self.variant = int(variant)

    def material_count(self, m: int) -> int:
        """Materials of model m's indexed stress coefficients (0: per-cell arrays)."""
        return lib().seidart_batch_material_count(self.handle, int(m))

    @staticmethod
    def num_variants() -> int:
        _declare()
        return lib().seidart_batch_num_variants()

    def _solver(self, m: int):
        return lib().seidart_batch_model(self.handle, m)

    def _set_fields(self, m, fields):
        arrs = [None if f is None else np.asfortranarray(f) for f in fields]
        rc = lib().seidart_solver_set_fields(self._solver(m), ptr_array(arrs))
        if rc != 0:
            raise SeidartError(rc, lib().seidart_last_error().decode())

    def step(self, n: int, chunk: int | None = None) -> None:
        _check(lib().seidart_batch_step(self.handle, int(n), int(chunk or n)))

    def sync(self) -> None:
        _check(lib().seidart_batch_sync(self.handle))

    @property
    def steps_done(self) -> int:
        return lib().seidart_batch_steps_done(self.handle)

    @property
    def launches(self) -> int:
        return lib().seidart_batch_launches(self.handle)

    @property
    def graph_launches(self) -> int:
        """Launches of the last step() that were CUDA graph replays."""
        return lib().seidart_batch_graph_launches(self.handle)

    def fields(self, m: int) -> list:
        out = self.problems[m].field_list()
        rc = lib().seidart_solver_get_fields(self._solver(m), ptr_array(out))
        if rc != 0:
            raise SeidartError(rc, lib().seidart_last_error().decode())
        return out

    def traces(self, m: int):
        p = self.problems[m]
        n = self.steps_done
        nrec = len(p.receiver_array())
        tr = np.zeros((n, 2, nrec))
        nrm = np.zeros(n)
        rc = lib().seidart_solver_traces(self._solver(m), tr.ctypes.data if nrec else None, nrm.ctypes.data)
        if rc != 0:
            raise SeidartError(rc, lib().seidart_last_error().decode())
        return tr, nrm

    def force_barrier_timeout(self, spin_limit: int = 1 << 16) -> int:
        """Run one step whose grid barrier can never complete (it expects one
        CTA more than the grid holds); returns the status code the bounded
        wait produced (SEIDART_ERR_TIMEOUT = -6)."""
        return lib().seidart_batch_force_timeout(self.handle, int(spin_limit))

    def close(self):
        if getattr(self, "handle", None):
            lib().seidart_batch_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
