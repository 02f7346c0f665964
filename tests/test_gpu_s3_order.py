"""Memory-order options of the FP32 3D step change nothing in the results:
read-once copies of the staged stress kernel with an L2 evict-first policy
(SEIDART_S3_L2HINT) and the velocity kernel walking its planes from the top
(SEIDART_S3_VREV) give fields, memories, traces and norms bit for bit equal
to the plain order, on a small grid with a stress source and on 352^3."""
import dataclasses

import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import models

pytestmark = pytest.mark.gpu

KEYS = ("SEIDART_S3_L2HINT", "SEIDART_S3_VREV", "SEIDART_S3_WAVE")


def _run(p, env, monkeypatch):
    for k in KEYS:
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    with sg.Solver(p, sg.FP32) as s:
        s.step(p.time_steps)
        s.sync()
        tr, nrm = s.traces()
        return {"fields": s.get_fields(), "memory": s.get_memory(), "traces": tr, "norms": nrm}


@pytest.mark.parametrize("case", ["small", "352cube"])
@pytest.mark.parametrize("env", [{"SEIDART_S3_L2HINT": "0", "SEIDART_S3_VREV": "1"},
                                 {"SEIDART_S3_L2HINT": "1", "SEIDART_S3_VREV": "0"},
                                 {"SEIDART_S3_L2HINT": "1", "SEIDART_S3_VREV": "1"}], ids=["vrev", "l2hint", "both"])
def test_memory_order_options_change_nothing(case, env, monkeypatch):
    if case == "small":
        p = models.seismic3_layers(n=48, cpml=8, nt=40, nlayers=3, nrec_side=6, rec_z=3, src_z=10)
        p = dataclasses.replace(p, src={"xx": 1e6 * p.src["z"], "z": p.src["z"]})
    else:
        p = models.seismic3_layers(n=320, cpml=16, nt=12, seed=2)
    base = _run(p, {"SEIDART_S3_L2HINT": "0", "SEIDART_S3_VREV": "0"}, monkeypatch)
    got = _run(p, env, monkeypatch)
    assert np.max(np.abs(base["traces"])) > 0
    assert np.array_equal(got["traces"], base["traces"])
    assert np.array_equal(got["norms"], base["norms"])
    for q in range(9):
        assert np.array_equal(got["fields"][q], base["fields"][q]), q
    if case == "small":
        for q in range(45):
            assert np.array_equal(got["memory"][q], base["memory"][q]), q
