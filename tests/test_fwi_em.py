"""Misfit gradient of the 2D electromagnetic solver (hand-written adjoint,
csrc/adjoint_em.cu driven by csrc/adjoint.cu).

CPU: the FP64 torch restatement used as gradient oracle reproduces
oracle.c's electromag2 traces, and its autograd gradient matches central
differences of oracle.c.
GPU: the adjoint step is the transpose of the forward step (dot-product
test); the gradient with respect to eps11, eps13, eps33, sig11, sig13,
sig33 matches the FP64 oracle gradient on a 64 x 64 instance and central
differences (relative perturbation 1e-4) of the FP64 misfit at 8 seeded
cells within 1e-3; the torch autograd wrapper returns it.
"""
from dataclasses import replace

import numpy as np
import pytest

GRAD_TOL = 1e-3
KEYS = ("e11", "e13", "e33", "s11", "s13", "s33")


def _case(n=64, cpml=10, nt=360, nshots=2, nrec=16, f0=4.0e8):
    """Start model: background eps = 4 (eps13 = 0.3), sigma = 1e-3 with a
    full tensor; true model: a Gaussian anomaly (+30% eps11, eps33, sigma
    x 3) between the sources and depth.  The misfit is far above the FP32
    rounding of the traces, so the FP32 gradient can be held to 1e-3."""
    from seidart_gpu import models
    from seidart_gpu.fwi import Shot, with_model
    p = models.electromag2_blocks(n=n, cpml=cpml, nt=nt, f0=f0, src=(n // 2, 8), nrec=nrec, rec_z=6, nblocks=0)
    shape = p.shape
    start = with_model(p, e13=np.full(shape, 0.3), s11=np.full(shape, 1e-3), s13=np.full(shape, 2e-4),
                       s33=np.full(shape, 1.5e-3))
    x = np.arange(shape[0])[:, None]
    z = np.arange(shape[1])[None, :]
    g = np.exp(-((x - (n // 2 + cpml)) ** 2 + (z - (n // 3 + cpml)) ** 2) / (2 * (n / 10) ** 2))
    true = with_model(start, e11=start.model["e11"] * (1 + 0.3 * g), e33=start.model["e33"] * (1 + 0.3 * g),
                      s11=start.model["s11"] * (1 + 2 * g), s33=start.model["s33"] * (1 + 2 * g))
    xs = np.linspace(n // 4, 3 * n // 4, nshots).astype(int)
    shots = [Shot(int(xx), 8, start.src["z"]) for xx in xs]
    return start, true, shots


def _shot_problem(p, shot):
    return replace(p, xind=shot.xind, zind=shot.zind, src={"z": shot.srcz})


def _oracle_observed(oracle, p, shots):
    return [oracle.run_oracle(_shot_problem(p, s))["traces"] for s in shots]


def _oracle_loss(oracle, p, shots, observed):
    return sum(0.5 * float(np.sum((oracle.run_oracle(_shot_problem(p, s))["traces"] - o) ** 2))
               for s, o in zip(shots, observed))


def _fd(oracle, start, shots, obs, key, cell):
    from seidart_gpu.fwi import with_model
    base = start.model[key]
    h = 1e-4 * abs(base[cell])
    plus, minus = base.copy(order="F"), base.copy(order="F")
    plus[cell] += h
    minus[cell] -= h
    return (_oracle_loss(oracle, with_model(start, **{key: plus}), shots, obs)
            - _oracle_loss(oracle, with_model(start, **{key: minus}), shots, obs)) / (2 * h)


# ------------------------------------------------------------------- CPU
def test_em_grad_oracle_forward_matches_c_oracle(oracle):
    torch = pytest.importorskip("torch")
    from oracle import grad_torch
    start, true, shots = _case(n=32, cpml=6, nt=150, nshots=1, nrec=8)
    p = _shot_problem(true, shots[0])
    ref = oracle.run_oracle(p)["traces"]
    m = {k: torch.tensor(v) for k, v in p.model.items()}
    tr = grad_torch.em2_forward_traces(m, p.dx, p.dz, p.dt, p.time_steps,
                                       (p.xind + p.cpml - 1, p.zind + p.cpml - 1), p.src["z"],
                                       np.asarray(p.receivers, dtype=np.int64)).numpy()
    assert np.max(np.abs(ref)) > 0
    assert np.linalg.norm(tr - ref) <= 1e-12 * np.linalg.norm(ref)


def test_em_grad_oracle_matches_finite_differences(oracle):
    pytest.importorskip("torch")
    from oracle import grad_torch
    start, true, shots = _case(n=32, cpml=6, nt=150, nshots=1, nrec=8)
    obs = _oracle_observed(oracle, true, shots)
    loss, g = grad_torch.em2_misfit_and_gradient(start, shots, obs)
    assert loss == pytest.approx(_oracle_loss(oracle, start, shots, obs), rel=1e-12)
    for key in ("e33", "s11", "e13"):
        a = np.abs(g[key])
        cell = np.unravel_index(np.argmax(a), a.shape)
        fd = _fd(oracle, start, shots, obs, key, cell)
        assert abs(fd - g[key][cell]) <= 1e-5 * abs(fd), (key, fd, g[key][cell])


# ------------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_em_adjoint_is_transpose_of_step():
    from seidart_gpu.fwi import NSTATE_EM, Fwi
    start, _, shots = _case(n=48, cpml=8, nt=20, nshots=1, nrec=4)
    rng = np.random.default_rng(5)
    n = start.ncell
    with Fwi(start, shots) as f:
        assert f.nstate == NSTATE_EM
        for trial in range(3):
            # fields of the size a GPR run carries (E ~ 1, H ~ E / 377)
            x = rng.standard_normal((NSTATE_EM, n)).astype(np.float32)
            x[2] *= 1e-3
            lam = rng.standard_normal((NSTATE_EM, n)).astype(np.float32)
            y = f.forward_step(x)
            z = f.adjoint_step(x, y, lam)
            lhs = float(np.dot(y.ravel().astype(np.float64), lam.ravel().astype(np.float64)))
            rhs = float(np.dot(x.ravel().astype(np.float64), z.ravel().astype(np.float64)))
            assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs)), (trial, lhs, rhs)


@pytest.fixture(scope="module")
def em64(oracle):
    pytest.importorskip("torch")
    from oracle import grad_torch
    start, true, shots = _case()
    obs = _oracle_observed(oracle, true, shots)
    loss, g = grad_torch.em2_misfit_and_gradient(start, shots, obs)
    return start, shots, obs, loss, g


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
def test_em_gradient_matches_fp64_oracle_gradient(em64):
    from seidart_gpu.fwi import Fwi
    start, shots, obs, loss64, g64 = em64
    with Fwi(start, shots, obs) as f:
        loss, g = f.gradient()
    assert abs(loss - loss64) <= 1e-3 * loss64
    for k in KEYS:
        assert _rel(g[k], g64[k]) <= GRAD_TOL, (k, _rel(g[k], g64[k]))


@pytest.mark.gpu
def test_em_gradient_matches_finite_differences(em64, oracle):
    from seidart_gpu.fwi import Fwi
    start, shots, obs, _, _ = em64
    with Fwi(start, shots, obs) as f:
        _, g = f.gradient()
    rng = np.random.default_rng(12)
    checked = 0
    for key, ncell in (("e11", 2), ("e33", 2), ("e13", 1), ("s11", 1), ("s33", 1), ("s13", 1)):
        a = np.abs(g[key])
        strong = np.argwhere(a >= 0.2 * a.max())
        for cell in strong[rng.choice(len(strong), size=ncell, replace=False)]:
            cell = tuple(cell)
            fd = _fd(oracle, start, shots, obs, key, cell)
            assert abs(g[key][cell] - fd) <= GRAD_TOL * abs(fd), (key, cell, g[key][cell], fd)
            checked += 1
    assert checked == 8


@pytest.mark.gpu
def test_em_torch_autograd_wrapper(em64):
    torch = pytest.importorskip("torch")
    from seidart_gpu.fwi import Fwi, electromag2_misfit
    start, shots, obs, _, _ = em64
    ts = [torch.tensor(start.model[k], requires_grad=True) for k in KEYS]
    loss = electromag2_misfit(*ts, start, shots, obs)
    (3.0 * loss).backward()
    with Fwi(start, shots, obs) as f:
        l2, g = f.gradient()
    assert float(loss.detach()) == pytest.approx(l2, rel=1e-13)
    for t, k in zip(ts, KEYS):
        assert np.array_equal(t.grad.numpy(), 3.0 * g[k])


@pytest.mark.gpu
def test_em_model_traces_match_solver():
    import seidart_gpu as sg
    from seidart_gpu.fwi import Fwi
    start, _, shots = _case(n=48, cpml=8, nt=80, nshots=2, nrec=6)
    with Fwi(start, shots) as f:
        tr = f.model_traces()
    for s, shot in enumerate(shots):
        ref = sg.run(_shot_problem(start, shot), sg.FP32)["traces"]
        assert np.array_equal(tr[s], ref)
