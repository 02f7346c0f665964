"""The fused FP32 3D step (both half-steps in one wavefront launch) and the
bounded device waits of the FP32 3D kernels.

* The fused step against the two-kernel step on the same problem: bit for
  bit against the one-cell velocity kernel (same arithmetic), within 1e-6
  of the cell-pair velocity kernel, and within 1e-4 of the CPU restatement;
  with a stress source, a grid whose planes hold more tiles than the GPU
  runs CTAs at once, and odd y/z sizes.
* Timeouts: the test hook of seidart_solver_set_wait arms one CTA's copy
  barrier with bytes no copy brings (and, in the fused step, one plane wait
  with a count no plane reaches).  Every copy still lands, the bounded wait
  runs out, the kernel returns, seidart_solver_sync reports
  SEIDART_ERR_TIMEOUT once, and the same solver then runs normal steps.
  Covered for the fused step, the staged stress kernel and the TMA
  z-marching stress kernel.  Nothing here faults or hangs the GPU: the
  waits that run out are on a barrier whose copies all complete.
"""
import dataclasses

import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import models
from seidart_gpu._lib import SeidartError

pytestmark = pytest.mark.gpu

TIMEOUT = -6  # SEIDART_ERR_TIMEOUT
WAVE = {"SEIDART_S3_WAVE": "1"}


def rel_l2(a, b):
    nb = np.linalg.norm(np.ravel(b))
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / (nb if nb > 0 else 1.0))


def _run(p, env, monkeypatch, nsteps=None):
    for k in ("SEIDART_S3_WAVE", "SEIDART_S3_VPAIR", "SEIDART_S3_STRESS"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    with sg.Solver(p, sg.FP32) as s:
        s.step(p.time_steps if nsteps is None else nsteps)
        s.sync()
        tr, nrm = s.traces()
        return {"fields": s.get_fields(), "memory": s.get_memory(), "traces": tr, "norms": nrm,
                "launches": s.launches}


def _cases():
    base = models.seismic3_layers(n=48, cpml=8, nt=60, nlayers=3, nrec_side=6, rec_z=3, src_z=10)
    src = base.src["z"]
    stress = dataclasses.replace(base, src={"xx": 1e6 * src, "yz": 3e5 * src, "z": src})
    odd = models.seismic3_layers(n=48, cpml=8, nt=40, nlayers=3, nrec_side=6, rec_z=3, src_z=10, ny=45, nz=43)
    return {"force": base, "stress_source": stress, "odd_yz": odd}


@pytest.mark.parametrize("case", ["force", "stress_source", "odd_yz"])
def test_wave_step_matches_two_kernel_step(case, monkeypatch, oracle):
    p = _cases()[case]
    assert p.nx % 4 == 0
    wave = _run(p, WAVE, monkeypatch)
    cell = _run(p, {"SEIDART_S3_WAVE": "0", "SEIDART_S3_VPAIR": "0"}, monkeypatch)
    pair = _run(p, {"SEIDART_S3_WAVE": "0"}, monkeypatch)
    assert wave["launches"] < cell["launches"]  # one launch replaced two
    assert np.max(np.abs(wave["traces"])) > 0
    for key in ("traces", "norms"):
        assert np.array_equal(wave[key], cell[key]), key
        assert rel_l2(wave[key], pair[key]) <= 1e-6, key
    for q in range(9):
        assert np.array_equal(wave["fields"][q], cell["fields"][q]), q
    for q in range(45):
        assert np.array_equal(wave["memory"][q], cell["memory"][q]), q
    ref = oracle.run_oracle(p)
    for q in range(9):
        assert rel_l2(wave["fields"][q], ref["fields"][q]) <= 1e-4, q
    assert rel_l2(wave["traces"], ref["traces"]) <= 1e-4


def test_wave_step_full_size_matches_two_kernel_step(monkeypatch):
    """352^3 (484 tiles per plane, more than the CTAs the GPU holds at once
    at 4 per SM): 20 steps of the fused step against the two-kernel step."""
    p = models.seismic3_layers(n=320, cpml=16, nt=20, seed=2)
    wave = _run(p, WAVE, monkeypatch)
    cell = _run(p, {"SEIDART_S3_WAVE": "0", "SEIDART_S3_VPAIR": "0"}, monkeypatch)
    assert np.array_equal(wave["traces"], cell["traces"])
    assert np.array_equal(wave["norms"], cell["norms"])
    for q in range(9):
        assert np.array_equal(wave["fields"][q], cell["fields"][q]), q


@pytest.mark.parametrize("env", [{"SEIDART_S3_WAVE": "1"}, {"SEIDART_S3_WAVE": "0"},
                                 {"SEIDART_S3_WAVE": "0", "SEIDART_S3_STRESS": "tma"}],
                         ids=["wave", "staged_stress", "tma_stress"])
def test_bounded_wait_timeout_reports_status(env, monkeypatch):
    p = models.seismic3_layers(n=48, cpml=8, nt=30, nlayers=3, nrec_side=6, rec_z=3, src_z=10)
    for k in ("SEIDART_S3_WAVE", "SEIDART_S3_VPAIR", "SEIDART_S3_STRESS"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    clean = _run(p, env, monkeypatch, nsteps=10)
    with sg.Solver(p, sg.FP32) as s:
        s.set_wait(2000, 16)          # one CTA's wait runs out
        s.step(2)
        with pytest.raises(SeidartError) as e:
            s.sync()
        assert e.value.code == TIMEOUT
        s.set_wait(1 << 20, 0)        # back to normal: the solver keeps working
        s.step(3)
        s.sync()
        tr, _ = s.traces()
        assert np.all(np.isfinite(tr))
    # a new solver on the same context still gives the clean result
    again = _run(p, env, monkeypatch, nsteps=10)
    assert np.array_equal(again["traces"], clean["traces"])
    for q in range(9):
        assert np.array_equal(again["fields"][q], clean["fields"][q]), q
