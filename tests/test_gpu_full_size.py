"""Full-size workloads on the GPU, checked through properties that do not
need an oracle run of that size.

* seismic3 at 320^3 + 16 CPML (352^3 cells, the benchmark workload):
  FP32 against FP64 within 1e-4 relative L2, the fast FP64 build against the
  exact one within 1e-12, stepping in chunks equal to stepping at once (bit
  for bit), and linearity in the source: doubling every source series
  doubles every field, memory, trace and norm (scaling by 2 commutes with
  rounding, so the FP64 run must match bit for bit and the FP32 run to
  within its subnormal far field).
* the same seismic3 workload for all 1500 steps of its configuration: FP32
  traces and final fields within 1e-4 relative L2 of the fast FP64 build
  (itself within 1e-12 of exact FP64, checked above and in the bench).
* seismic2 two-layer (256^2 + 20 CPML, 2000 steps, the 2D elastic
  configuration): the exact FP64 build bit for bit against the CPU
  restatement over all 2000 steps.
* electromag2 at 1024^2 + 20 CPML (1064^2 cells) for the full 4000 steps:
  FP32 against FP64 and fast FP64 against FP64.
"""
import dataclasses

import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import models

pytestmark = pytest.mark.gpu

NSTEPS_3D = 30


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="module")
def cube():
    return models.seismic3_layers(n=320, cpml=16, nt=NSTEPS_3D, seed=2)


def _run(p, prec, chunks=None):
    with sg.Solver(p, prec) as s:
        for n in (chunks or [p.time_steps]):
            s.step(n)
        s.sync()
        tr, nrm = s.traces()
        return {"fields": s.get_fields(), "traces": tr, "norms": nrm}


def test_seismic3_full_size_precisions(cube):
    g64 = _run(cube, sg.FP64)
    g32 = _run(cube, sg.FP32)
    gx = _run(cube, sg.FP64_FAST)
    assert np.max(np.abs(g64["traces"])) > 0
    assert rel_l2(g32["traces"], g64["traces"]) <= 1e-4
    assert rel_l2(gx["traces"], g64["traces"]) <= 1e-12
    for q in range(9):
        assert rel_l2(g32["fields"][q], g64["fields"][q]) <= 1e-4, q
        assert rel_l2(gx["fields"][q], g64["fields"][q]) <= 1e-12, q


def test_seismic3_full_size_chunking(cube):
    a = _run(cube, sg.FP32)
    b = _run(cube, sg.FP32, chunks=[7, 1, NSTEPS_3D - 8])
    assert np.array_equal(a["traces"], b["traces"]) and np.array_equal(a["norms"], b["norms"])
    for q in range(9):
        assert np.array_equal(a["fields"][q], b["fields"][q]), q


def test_seismic3_full_size_linearity(cube):
    twice = dataclasses.replace(cube, src={k: 2.0 * v for k, v in cube.src.items()})
    a64, b64 = _run(cube, sg.FP64), _run(twice, sg.FP64)
    assert np.array_equal(2.0 * a64["traces"], b64["traces"])
    assert np.array_equal(2.0 * a64["norms"], b64["norms"])
    for q in range(9):
        assert np.array_equal(2.0 * a64["fields"][q], b64["fields"][q]), q
    a32, b32 = _run(cube, sg.FP32), _run(twice, sg.FP32)
    assert rel_l2(b32["traces"], 2.0 * a32["traces"]) <= 1e-6
    for q in range(9):
        assert rel_l2(b32["fields"][q], 2.0 * a32["fields"][q]) <= 1e-6, q


def test_seismic3_full_length_fp32_vs_fp64():
    """All 1500 steps of the 3D configuration from the zero state: by then the
    wavefront from the centre-top source has crossed the receiver grid and
    reached the CPML, so traces and fields carry the whole propagation."""
    p = models.seismic3_layers(n=320, cpml=16, nt=1500, seed=2)
    g32 = _run(p, sg.FP32)
    gx = _run(p, sg.FP64_FAST)
    assert np.max(np.abs(gx["traces"])) > 0
    assert rel_l2(g32["traces"], gx["traces"]) <= 1e-4
    assert rel_l2(g32["norms"], gx["norms"]) <= 1e-4
    for q in range(9):
        assert rel_l2(g32["fields"][q], gx["fields"][q]) <= 1e-4, q


def test_seismic2_config0_full_length_bit_exact(oracle):
    """The 2D elastic configuration for all 2000 steps: exact FP64 on the GPU
    equals the CPU restatement bit for bit (fields, CPML memories, traces,
    norms)."""
    p = models.seismic2_two_layer()  # 256^2 + 20 CPML, 2000 steps
    ref = oracle.run_oracle(p)
    got = sg.run(p, sg.FP64)
    assert np.max(np.abs(ref["traces"])) > 0
    assert np.array_equal(got["traces"], ref["traces"])
    assert np.array_equal(got["norms"], ref["norms"])
    for a, b in zip(got["fields"], ref["fields"]):
        assert np.array_equal(a, b)
    for a, b in zip(got["memory"], ref["memory"]):
        assert np.array_equal(a, b)


def test_electromag2_full_size_full_length():
    p = models.electromag2_blocks()  # 1024^2 + 20 CPML, 12 blocks, 4000 steps
    g64 = _run(p, sg.FP64)
    g32 = _run(p, sg.FP32)
    gx = _run(p, sg.FP64_FAST)
    assert np.max(np.abs(g64["traces"])) > 0
    assert rel_l2(g32["traces"], g64["traces"]) <= 1e-4
    assert rel_l2(gx["traces"], g64["traces"]) <= 1e-12


def test_ragged_batch_full_size():
    """The 64-model ragged batch (nx, nz in [256, 1024] + 20 CPML, 29.4 M
    cells) for 200 steps in chunks, against single-model FP32 runs of a
    sample of its models (smallest, largest, two in between)."""
    from seidart_gpu.batch import Batch
    ps = models.batch_layered_vti(nmodels=64, nt=200)
    with Batch(ps, autotune=True, trial_steps=8) as b:
        b.step(50, chunk=25)
        b.step(150, chunk=100)
        b.sync()
        order = np.argsort([p.ncell for p in ps])
        for m in (order[0], order[21], order[42], order[-1]):
            single = sg.run(ps[m], sg.FP32)
            tr, nrm = b.traces(m)
            assert np.max(np.abs(single["fields"][1])) > 0
            assert rel_l2(tr, single["traces"]) <= 1e-6, m
            assert rel_l2(nrm, single["norms"]) <= 1e-6, m
            f = b.fields(m)
            for q in range(5):
                assert rel_l2(f[q], single["fields"][q]) <= 1e-6, (m, q)
