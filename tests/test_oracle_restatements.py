"""The C restatement (oracle.c) against the independent numpy restatement.

Both follow src/fortran/cpmlfdtd.f08 with the same expression trees in IEEE
double without FMA, so every field, CPML memory array, receiver sample and
norm must agree bit for bit.  A transcription slip in either shows up here.
"""
import numpy as np
import pytest

from oracle import restate_np
from seidart_gpu import models


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.array_equal(a, b), f"max |diff| = {np.max(np.abs(a - b))}"


@pytest.mark.parametrize("density", ["harmonic", "geometric", "arithmetic", "none"])
def test_seismic2_c_equals_numpy(oracle, density):
    p = models.seismic2_two_layer(n=40, cpml=6, nt=60, src=(20, 8), nrec=8, rec_z=4, density=density, gamma=7.0)
    # a stress source as well, so every injection term is exercised
    p.src["xx"] = 0.3 * p.src["z"]
    p.src["xz"] = -0.2 * p.src["z"]
    p.src["zz"] = 0.1 * p.src["z"]
    c = oracle.run_oracle(p)
    n = restate_np.seismic2(p, p.time_steps)
    for a, b in zip(c["fields"], n["fields"]):
        _same(a, b)
    for a, b in zip(c["memory"], n["memory"]):
        _same(a, b)
    _same(c["traces"], n["traces"])
    _same(c["norms"], n["norms"])


def test_electromag2_c_equals_numpy(oracle):
    p = models.electromag2_blocks(n=48, cpml=6, nt=80, src=(24, 8), nrec=8, rec_z=5, nblocks=4)
    # an off-diagonal permittivity and conductivity exercise every coefficient
    p.model["e13"][:] = 0.5
    p.model["s13"][:] = 1e-3
    c = oracle.run_oracle(p)
    n = restate_np.electromag2(p, p.time_steps)
    for a, b in zip(c["fields"], n["fields"]):
        _same(a, b)
    for a, b in zip(c["memory"], n["memory"]):
        _same(a, b)
    _same(c["traces"], n["traces"])
    _same(c["norms"], n["norms"])


def test_seismic3_c_equals_numpy(oracle):
    p = models.seismic3_layers(n=14, cpml=4, nt=25, nlayers=3, nrec_side=3, rec_z=2, src_z=5)
    for k in ("xx", "xy", "xz", "yy", "yz", "zz"):
        p.src[k] = 0.1 * p.src["z"]
    p.src["x"] = 0.5 * p.src["z"]
    p.src["y"] = -0.5 * p.src["z"]
    c = oracle.run_oracle(p)
    n = restate_np.seismic3(p, p.time_steps)
    for a, b in zip(c["fields"], n["fields"]):
        _same(a, b)
    for a, b in zip(c["memory"], n["memory"]):
        _same(a, b)
    _same(c["traces"], n["traces"])
    _same(c["norms"], n["norms"])


def test_electromag3_c_equals_numpy(oracle):
    p = models.electromag3_blocks(n=14, cpml=4, nt=30, nblocks=3, nrec_side=3)
    # a full conductivity tensor exercises every coupling term
    for c in ("s12", "s13", "s23"):
        p.model[c][:] = 2e-4
    p.model["s11"][:] = 3e-3
    c = oracle.run_oracle(p)
    n = restate_np.electromag3(p, p.time_steps)
    for a, b in zip(c["fields"], n["fields"]):
        _same(a, b)
    for a, b in zip(c["memory"], n["memory"]):
        _same(a, b)
    _same(c["traces"], n["traces"])
    _same(c["norms"], n["norms"])
    assert np.max(np.abs(c["traces"])) > 0
