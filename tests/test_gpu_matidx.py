"""Layouts of the FP32 3D stress kernel that change what it reads, not what
it computes.

Material-indexed coefficients: a model whose 21 C_ij and 6 attenuation
arrays hold few distinct tuples (layers, or any model expanded from a
material image) runs with one byte per cell and a table of FP32 tuples;
fields, memories, traces and norms equal the per-cell layout
(SEIDART_S3_MATIDX=0) bit for bit.  A model with a distinct tuple per cell,
or more than 32 tuples, keeps the per-cell layout.

Merged C-PML memories: the stress loops' 36 memories held as 21 (the loops
that share a derivative stencil and its coefficients share the memory);
the results and the 36 memories rebuilt on read-back equal the 36-array
layout (SEIDART_S3_MERGE=0) bit for bit.

Indexed C-PML coefficients: the six C-PML grids read as one byte per cell
and a table when they hold at most 64 tuples; bit for bit the grids
(SEIDART_S3_CPMLIDX=0), which more tuples keep."""
import dataclasses

import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import models

pytestmark = pytest.mark.gpu


def _run(p, indexed, monkeypatch, memory=True, merged=True, cpmlidx=True):
    monkeypatch.setenv("SEIDART_S3_MATIDX", "1" if indexed else "0")
    monkeypatch.setenv("SEIDART_S3_MERGE", "1" if merged else "0")
    monkeypatch.setenv("SEIDART_S3_CPMLIDX", "1" if cpmlidx else "0")
    with sg.Solver(p, sg.FP32) as s:
        nmat = s.material_count()
        ncpml = s.cpml_tuples()
        s.step(p.time_steps)
        s.sync()
        tr, nrm = s.traces()
        out = {"fields": s.get_fields(), "traces": tr, "norms": nrm, "nmat": nmat, "ncpml": ncpml}
        if memory:
            out["memory"] = s.get_memory()
        return out


def _same(a, b, memory=True):
    assert np.max(np.abs(b["traces"])) > 0
    assert np.array_equal(a["traces"], b["traces"])
    assert np.array_equal(a["norms"], b["norms"])
    for q in range(9):
        assert np.array_equal(a["fields"][q], b["fields"][q]), q
    if memory:
        for q in range(45):
            assert np.array_equal(a["memory"][q], b["memory"][q]), q


def test_layered_model_is_indexed_and_bit_identical(monkeypatch):
    p = models.seismic3_layers(n=48, cpml=8, nt=40, nlayers=3, nrec_side=6, rec_z=3, src_z=10)
    # a stress source as well, so the source cells' path is covered
    p = dataclasses.replace(p, src={"xx": 1e6 * p.src["z"], "z": p.src["z"]})
    got = _run(p, True, monkeypatch)
    base = _run(p, False, monkeypatch)
    assert got["nmat"] == 3 and base["nmat"] == 0
    _same(got, base)


def test_thirty_two_materials_indexed_thirty_three_not(monkeypatch):
    """Up to 32 tuples take the indexed layout; one more keeps the per-cell
    arrays.  Extra materials are blocks of perturbed c11 inside the grid."""
    p = models.seismic3_layers(n=40, cpml=8, nt=20, nlayers=2, nrec_side=4, rec_z=3, src_z=10)
    for extra, want in ((30, 32), (31, 0)):
        model = {k: v.copy() for k, v in p.model.items()}
        for b in range(extra):
            x0 = 8 + 4 * (b % 8)
            y0 = 8 + 8 * (b // 8)
            model["c11"][x0:x0 + 3, y0:y0 + 3, 20:23] *= 1.0 + 0.001 * (b + 1)
        q = dataclasses.replace(p, model=model)
        got = _run(q, True, monkeypatch, memory=False)
        assert got["nmat"] == want, (extra, got["nmat"])
        base = _run(q, False, monkeypatch, memory=False)
        _same(got, base, memory=False)


def test_per_cell_model_keeps_the_per_cell_layout(monkeypatch):
    p = models.seismic3_layers(n=40, cpml=8, nt=20, nlayers=2, nrec_side=4, rec_z=3, src_z=10)
    rng = np.random.default_rng(5)
    model = {k: v.copy() for k, v in p.model.items()}
    model["c33"] = np.asfortranarray(model["c33"] * (1.0 + 1e-3 * rng.random(model["c33"].shape)))
    q = dataclasses.replace(p, model=model)
    got = _run(q, True, monkeypatch, memory=False)
    assert got["nmat"] == 0


def test_full_size_indexed_matches_per_cell(monkeypatch):
    p = models.seismic3_layers(n=320, cpml=16, nt=12, seed=2)
    got = _run(p, True, monkeypatch, memory=False)
    base = _run(p, False, monkeypatch, memory=False)
    assert got["nmat"] == 5
    _same(got, base, memory=False)


@pytest.mark.parametrize("indexed", [True, False])
def test_merged_memories_equal_the_36_array_layout(indexed, monkeypatch):
    """A grid small enough that every cell is a C-PML cell near some face, a
    stress source, and all four loops' boundary rows: fields, traces, norms
    and the 36 stress-loop memories (rebuilt from the 21 merged ones)."""
    p = models.seismic3_layers(n=24, cpml=8, nt=40, nlayers=2, nrec_side=4, rec_z=3, src_z=6)
    p = dataclasses.replace(p, src={"xx": 1e6 * p.src["z"], "yz": -5e5 * p.src["z"], "z": p.src["z"]})
    got = _run(p, indexed, monkeypatch, merged=True)
    base = _run(p, indexed, monkeypatch, merged=False)
    _same(got, base)
    assert max(np.max(np.abs(m)) for m in base["memory"][:36]) > 0


def test_cpml_index_is_bit_identical(monkeypatch):
    p = models.seismic3_layers(n=40, cpml=8, nt=40, nlayers=2, nrec_side=4, rec_z=3, src_z=6)
    got = _run(p, True, monkeypatch, cpmlidx=True)
    base = _run(p, True, monkeypatch, cpmlidx=False)
    assert got["ncpml"] > 0 and base["ncpml"] == 0
    _same(got, base)


def test_many_cpml_tuples_keep_the_grids(monkeypatch):
    p = models.seismic3_layers(n=40, cpml=8, nt=10, nlayers=2, nrec_side=4, rec_z=3, src_z=6)
    rng = np.random.default_rng(3)
    model = {k: v.copy() for k, v in p.model.items()}
    a = model["acoef"]
    model["acoef"] = np.asfortranarray(np.where(a != 0, a * (1.0 + 1e-3 * rng.random(a.shape)), a))
    q = dataclasses.replace(p, model=model)
    got = _run(q, True, monkeypatch, memory=False)
    assert got["ncpml"] == 0
