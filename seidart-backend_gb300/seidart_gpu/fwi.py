"""Misfit gradients of the 2D solvers (full-waveform inversion).

:class:`Fwi` binds ``seidart_fwi_*`` of the C ABI: shots with their own
source positions and series, a common receiver set and observed traces per
shot.  :meth:`Fwi.gradient` returns the L2 receiver misfit

    L = 1/2 sum_shots sum_steps sum_receivers (u_x - d_x)^2 + (u_z - d_z)^2

of the FP32 solver (u = vx, vz for seismic2, Ex, Ez for electromag2) and its
gradient on the padded grid from a hand-written discrete adjoint
(csrc/adjoint.cu, csrc/adjoint_em.cu): FP32 fields, FP64 gradient
accumulation, sqrt(nt) checkpointing with recomputation.  seismic2 shots are
vertical forces and the gradient is dL/d{c11, c13, c33, c55, rho};
electromag2 shots drive Ez and the gradient is dL/d{e11, e13, e33, s11, s13,
s33} (relative permittivity and conductivity, as in e11.dat ... s33.dat).
``seismic2_misfit`` and ``electromag2_misfit`` wrap them as
``torch.autograd.Function``s; torch is imported only there.  The reference
(SeidarT-Backend) has forward models only; the forward operators
differentiated here are its seismic2 and electromag2 time loops
(src/fortran/cpmlfdtd.f08:311-576, :2519-2748) as computed by the FP32
solvers.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, replace

import numpy as np

from ._lib import ELECTROMAG2, SEISMIC2, SeidartError, UnstableError, lib, ptr_array
from .api import Problem

GRAD_KEYS = ("c11", "c13", "c33", "c55", "rho")
GRAD_KEYS_FULL = GRAD_KEYS + ("c15", "c35")  # seismic2 with the full 2D tensor
GRAD_KEYS_EM = ("e11", "e13", "e33", "s11", "s13", "s33")
NSTATE = 17     # vx vz sigmaxx sigmazz sigmaxz + 12 memory arrays
NSTATE_EM = 7   # Ex Ez Hy + 4 memory arrays


def grad_keys(family: int, full_tensor: bool = False) -> tuple:
    if family == ELECTROMAG2:
        return GRAD_KEYS_EM
    return GRAD_KEYS_FULL if full_tensor else GRAD_KEYS

_DECL = False


def _declare():
    global _DECL
    if _DECL:
        return
    L = lib()
    vp, i = C.c_void_p, C.c_int
    sig = {
        "seidart_fwi_create": (i, [C.POINTER(vp), vp, vp, i, vp, i, vp, vp, vp, i, vp, vp, i]),
        "seidart_fwi_create_family": (i, [C.POINTER(vp), i, vp, vp, i, vp, i, vp, vp, vp, i, vp, vp, i]),
        "seidart_fwi_gradient": (i, [vp, vp, vp]),
        "seidart_fwi_model_traces": (i, [vp, vp]),
        "seidart_fwi_forward_step_host": (i, [vp, vp]),
        "seidart_fwi_adjoint_step_host": (i, [vp, vp, vp, vp]),
        "seidart_fwi_launches": (C.c_longlong, [vp]),
        "seidart_fwi_set_full_tensor": (i, [vp, i]),
        "seidart_fwi_checkpointing": (i, [vp, C.POINTER(i), C.POINTER(i)]),
        "seidart_fwi_destroy": (i, [vp]),
        "seidart_fwi_last_error": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    _DECL = True


def _check(rc: int) -> None:
    if rc != 0:
        msg = lib().seidart_fwi_last_error().decode(errors="replace")
        raise (UnstableError if rc == -3 else SeidartError)(rc, msg)


@dataclass
class Shot:
    """Source of one shot (seismic2: vertical force; electromag2: Ez
    source): interior indices as in Problem, series of time_steps samples."""
    xind: int
    zind: int
    srcz: np.ndarray


class Fwi:
    """Misfit and gradient of one 2D model (seismic2 or electromag2) over
    several shots."""

    def __init__(self, problem: Problem, shots: list[Shot], observed=None, checkpoint_every: int = 0,
                 full_tensor: bool = False):
        if problem.family not in (SEISMIC2, ELECTROMAG2):
            raise ValueError("the adjoint covers the 2D solvers seismic2 and electromag2")
        _declare()
        self.problem = problem
        self.shots = shots
        self.nshots = len(shots)
        self.nt = problem.time_steps
        rec = problem.receiver_array()
        self.nrec = len(rec)
        self._rec = rec
        self._model = problem.model_list()
        self._src = [np.ascontiguousarray(s.srcz, dtype=np.float64) for s in shots]
        for s in self._src:
            if s.shape != (self.nt,):
                raise ValueError(f"each shot needs {self.nt} source samples")
        shape = (self.nt, 2, self.nrec)
        if observed is None:
            self._obs = [None] * self.nshots
        else:
            self._obs = [np.ascontiguousarray(o, dtype=np.float64).reshape(shape) for o in observed]
        xs = np.array([s.xind for s in shots], dtype=np.int32)
        zs = np.array([s.zind for s in shots], dtype=np.int32)
        h = C.c_void_p()
        if full_tensor and problem.family != SEISMIC2:
            raise ValueError("full_tensor is for seismic2 (dL/dc15 and dL/dc35)")
        self.keys = grad_keys(problem.family, full_tensor)
        self.nstate = NSTATE_EM if problem.family == ELECTROMAG2 else NSTATE
        _check(lib().seidart_fwi_create_family(
            C.byref(h), problem.family, C.byref(problem.domain()), C.byref(problem.source()), problem.density_code(),
            ptr_array(self._model), self.nshots, xs.ctypes.data, zs.ctypes.data, ptr_array(self._src),
            self.nrec, rec.ctypes.data if self.nrec else None, ptr_array(self._obs), int(checkpoint_every)))
        self.handle = h
        if full_tensor:
            _check(lib().seidart_fwi_set_full_tensor(h, 1))

    # ---------------------------------------------------------------- compute
    def gradient(self) -> tuple[float, dict]:
        """(L, {key: dL/dm on the padded (nx, nz) grid}) with the keys of
        :func:`grad_keys` for the problem's family."""
        loss = C.c_double()
        n = self.problem.ncell
        g = np.zeros(len(self.keys) * n, dtype=np.float64)
        _check(lib().seidart_fwi_gradient(self.handle, C.byref(loss), g.ctypes.data))
        shape = self.problem.shape
        return loss.value, {k: g[q * n:(q + 1) * n].reshape(shape, order="F") for q, k in enumerate(self.keys)}

    def loss(self) -> float:
        loss = C.c_double()
        _check(lib().seidart_fwi_gradient(self.handle, C.byref(loss), None))
        return loss.value

    def model_traces(self) -> np.ndarray:
        """Synthetic traces [nshots][nt][2][nrec] of the current model (FP32 solver)."""
        out = np.zeros((self.nshots, self.nt, 2, self.nrec), dtype=np.float64)
        _check(lib().seidart_fwi_model_traces(self.handle, out.ctypes.data))
        return out

    def forward_step(self, x: np.ndarray) -> np.ndarray:
        """One step (source off) of an [nstate][ncell] FP32 state; returns the new state."""
        y = np.ascontiguousarray(x, dtype=np.float32).copy()
        _check(lib().seidart_fwi_forward_step_host(self.handle, y.ctypes.data))
        return y

    def adjoint_step(self, xprev: np.ndarray, xcur: np.ndarray, lam: np.ndarray) -> np.ndarray:
        """Transpose of one step applied to the adjoint state ``lam``."""
        xp = np.ascontiguousarray(xprev, dtype=np.float32)
        xc = np.ascontiguousarray(xcur, dtype=np.float32)
        out = np.ascontiguousarray(lam, dtype=np.float32).copy()
        _check(lib().seidart_fwi_adjoint_step_host(self.handle, xp.ctypes.data, xc.ctypes.data, out.ctypes.data))
        return out

    @property
    def launches(self) -> int:
        return lib().seidart_fwi_launches(self.handle)

    @property
    def checkpointing(self) -> tuple[int, int]:
        every, count = C.c_int(), C.c_int()
        _check(lib().seidart_fwi_checkpointing(self.handle, C.byref(every), C.byref(count)))
        return every.value, count.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().seidart_fwi_destroy(self.handle)
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


def with_model(problem: Problem, **arrays) -> Problem:
    """Copy of ``problem`` with some model arrays replaced."""
    model = dict(problem.model)
    for k, v in arrays.items():
        model[k] = np.asfortranarray(v, dtype=np.float64)
    return replace(problem, model=model)


def _torch_function():
    import torch

    class Seismic2Misfit(torch.autograd.Function):
        """L(c11, c13, c33, c55, rho) with the adjoint gradient as backward.

        forward(c11, c13, c33, c55, rho, problem, shots, observed) takes the
        five model grids as (nx, nz) tensors (any device; they are read as
        FP64 on the host) and returns the scalar misfit; the gradient is
        computed together with the loss (one forward, one checkpointed
        adjoint sweep) and scaled by grad_output in backward."""

        @staticmethod
        def forward(ctx, c11, c13, c33, c55, rho, problem, shots, observed, checkpoint_every=0):
            arrays = {k: t.detach().to("cpu", torch.float64).numpy() for k, t in
                      zip(GRAD_KEYS, (c11, c13, c33, c55, rho))}
            with Fwi(with_model(problem, **arrays), shots, observed, checkpoint_every) as f:
                loss, grads = f.gradient()
            ctx.save_for_backward(*[torch.from_numpy(np.ascontiguousarray(grads[k])).to(t.device, t.dtype)
                                    for k, t in zip(GRAD_KEYS, (c11, c13, c33, c55, rho))])
            return torch.tensor(loss, dtype=torch.float64, device=c11.device)

        @staticmethod
        def backward(ctx, gout):
            return tuple(gout.to(g.dtype) * g for g in ctx.saved_tensors) + (None, None, None, None)

    class Electromag2Misfit(torch.autograd.Function):
        """L(e11, e13, e33, s11, s13, s33) of an electromag2 problem with the
        adjoint gradient as backward (same contract as Seismic2Misfit)."""

        @staticmethod
        def forward(ctx, e11, e13, e33, s11, s13, s33, problem, shots, observed, checkpoint_every=0):
            ts = (e11, e13, e33, s11, s13, s33)
            arrays = {k: t.detach().to("cpu", torch.float64).numpy() for k, t in zip(GRAD_KEYS_EM, ts)}
            with Fwi(with_model(problem, **arrays), shots, observed, checkpoint_every) as f:
                loss, grads = f.gradient()
            ctx.save_for_backward(*[torch.from_numpy(np.ascontiguousarray(grads[k])).to(t.device, t.dtype)
                                    for k, t in zip(GRAD_KEYS_EM, ts)])
            return torch.tensor(loss, dtype=torch.float64, device=e11.device)

        @staticmethod
        def backward(ctx, gout):
            return tuple(gout.to(g.dtype) * g for g in ctx.saved_tensors) + (None, None, None, None)

    return Seismic2Misfit, Electromag2Misfit


_MISFIT = None


def _functions():
    global _MISFIT
    if _MISFIT is None:
        _MISFIT = _torch_function()
    return _MISFIT


def seismic2_misfit(c11, c13, c33, c55, rho, problem: Problem, shots: list[Shot], observed, checkpoint_every: int = 0):
    """Differentiable misfit: ``seismic2_misfit(...).backward()`` fills the
    ``.grad`` of the five model tensors."""
    return _functions()[0].apply(c11, c13, c33, c55, rho, problem, shots, observed, checkpoint_every)


def electromag2_misfit(e11, e13, e33, s11, s13, s33, problem: Problem, shots: list[Shot], observed,
                       checkpoint_every: int = 0):
    """Differentiable electromag2 misfit: ``.backward()`` fills the ``.grad``
    of the six permittivity and conductivity tensors."""
    return _functions()[1].apply(e11, e13, e33, s11, s13, s33, problem, shots, observed, checkpoint_every)
