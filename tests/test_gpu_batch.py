"""Ragged batch of 2D elastic models in one persistent cooperative launch."""
import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import models
from seidart_gpu.batch import Batch

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()) / max(np.linalg.norm(np.asarray(b).ravel()), 1e-300)


def small_batch(nt=60):
    return models.batch_layered_vti(nmodels=5, nt=nt, cpml=6, nmin=24, nmax=88, step=8, nrec=6, seed=11)


def test_batch_matches_single_model_runs(oracle):
    probs = small_batch()
    # one model with a stress source as well
    probs[2].src["xx"] = 0.3 * probs[2].src["z"]
    probs[2].src["xz"] = -0.2 * probs[2].src["z"]
    with Batch(probs, autotune=True, trial_steps=4) as b:
        assert b.tuning and len(b.tuning) >= 5
        b.step(25, chunk=10)
        # three chunks (10, 10, 5 steps): each a replay of a captured graph
        # holding one persistent launch
        assert b.launches == 3 and b.graph_launches == 3
        b.step(probs[0].time_steps - 25)
        b.sync()
        for m, p in enumerate(probs):
            single = sg.run(p, sg.FP32)
            tr, nrm = b.traces(m)
            f = b.fields(m)
            assert rel_l2(tr, single["traces"]) <= 1e-6
            for q in range(5):
                assert rel_l2(f[q], single["fields"][q]) <= 1e-6
            o = oracle.run_oracle(p)
            assert rel_l2(tr, o["traces"]) <= 1e-4
            assert rel_l2(nrm, o["norms"]) <= 1e-4


@pytest.mark.parametrize("variant", range(14))
def test_every_kernel_variant_matches_single_runs(variant):
    if variant >= Batch.num_variants():
        pytest.skip("variant not built")
    probs = small_batch(nt=40)
    probs[1].src["zz"] = 0.25 * probs[1].src["z"]
    with Batch(probs, autotune=False) as b:
        b.set_config(variant, 1)
        b.step(15, chunk=7)
        b.step(probs[0].time_steps - 15)
        b.sync()
        for m, p in enumerate(probs):
            single = sg.run(p, sg.FP32)
            tr, nrm = b.traces(m)
            assert rel_l2(tr, single["traces"]) <= 1e-6, (variant, m)
            assert rel_l2(nrm, single["norms"]) <= 1e-6, (variant, m)
            # final state in the solver's arrays (the fused walk double buffers
            # it and copies an odd-length launch's result back)
            f = b.fields(m)
            for q in range(5):
                assert rel_l2(f[q], single["fields"][q]) <= 1e-6, (variant, m, q)


def test_bounded_barrier_timeout_reports_status():
    """A barrier that can never complete gives up within its spin budget;
    the host sees SEIDART_ERR_TIMEOUT and the context stays usable."""
    probs = small_batch(nt=10)
    with Batch(probs, autotune=False) as b:
        assert b.force_barrier_timeout(spin_limit=1 << 14) == -6
    # the device still runs work afterwards
    with Batch(small_batch(nt=10), autotune=False) as b2:
        b2.step(10)
        b2.sync()


def test_sharded_batch_covers_every_model_once():
    """Two ranks' shares of one ragged batch (built one after the other on
    this GPU; the shares never wait on each other) reproduce every model."""
    from seidart_gpu.distributed import sharded_batch
    probs = small_batch(nt=30)
    seen = []
    for rank in range(2):
        b = sharded_batch(probs, rank, 2, autotune=False)
        with b:
            b.step(probs[0].time_steps)
            b.sync()
            for k in range(len(probs[rank::2])):
                m = rank + 2 * k
                single = sg.run(probs[m], sg.FP32)
                tr, _ = b.traces(k)
                assert rel_l2(tr, single["traces"]) <= 1e-6, m
                seen.append(m)
    assert sorted(seen) == list(range(len(probs)))


def test_material_indexed_batch_is_bit_identical(monkeypatch):
    """Layered models walk with one material byte per cell and a table of
    their stress-coefficient tuples; the traces, norms and fields equal the
    walk over per-cell arrays (SEIDART_BATCH_MATIDX=0) bit for bit, for the
    two-phase and the fused walks."""
    probs = small_batch(nt=40)
    probs[1].src["zz"] = 0.25 * probs[1].src["z"]
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("SEIDART_BATCH_MATIDX", flag)
        for variant in (11, Batch.num_variants() - 1):
            with Batch(probs, autotune=False) as b:
                mats = [b.material_count(m) for m in range(len(probs))]
                b.set_config(variant, 1)
                b.step(15, chunk=7)
                b.step(probs[0].time_steps - 15)
                b.sync()
                out[flag, variant] = (mats, [b.traces(m) for m in range(len(probs))],
                                      [b.fields(m) for m in range(len(probs))])
    for variant in (11, Batch.num_variants() - 1):
        mi, tri, fi = out["1", variant]
        mp, trp, fp = out["0", variant]
        assert all(m > 0 for m in mi) and all(m == 0 for m in mp)
        for m in range(len(probs)):
            assert np.array_equal(tri[m][0], trp[m][0]) and np.array_equal(tri[m][1], trp[m][1])
            for q in range(5):
                assert np.array_equal(fi[m][q], fp[m][q]), (variant, m, q)


@pytest.mark.parametrize("variant", [1, 11, 12])
def test_mixed_density_rules_use_the_generic_kernels(variant):
    """A batch whose models average density differently runs the kernels that
    read each model's rule at run time (a batch of one rule runs kernels
    compiled for it); both match single-model runs."""
    import dataclasses
    probs = small_batch(nt=30)
    probs = [dataclasses.replace(p, density=rule) for p, rule in
             zip(probs, ("harmonic", "arithmetic", "geometric", "none", "arithmetic"))]
    with Batch(probs, autotune=False) as b:
        b.set_config(variant, 1)
        b.step(probs[0].time_steps)
        b.sync()
        for m, p in enumerate(probs):
            single = sg.run(p, sg.FP32)
            tr, nrm = b.traces(m)
            assert rel_l2(tr, single["traces"]) <= 1e-6, (variant, m)
            assert rel_l2(nrm, single["norms"]) <= 1e-6, (variant, m)
