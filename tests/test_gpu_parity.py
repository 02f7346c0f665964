"""GPU solvers (through the C ABI) against the CPU restatement of the reference.

FP64 path: every field, CPML memory array, receiver sample and max-norm must
equal the oracle's exactly (the kernels keep the reference's expression
trees, --fmad=false).  FP32 path: relative L2 error against the FP64 oracle
at most FP32_TOL on fields and traces.
"""
import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import models

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4  # relative L2 of FP32 results against the FP64 oracle


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    return np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0)


def assert_exact(g, o):
    for name in ("fields", "memory"):
        for q, (a, b) in enumerate(zip(g[name], o[name])):
            assert np.array_equal(a, b), f"{name}[{q}] max |diff| {np.max(np.abs(a - b))}"
    assert np.array_equal(g["traces"], o["traces"]), f"traces max |diff| {np.max(np.abs(g['traces'] - o['traces']))}"
    assert np.array_equal(g["norms"], o["norms"]), "norms differ"


def small_problems():
    p1 = models.seismic2_two_layer(n=64, cpml=10, nt=150, src=(32, 12), nrec=16, rec_z=6, gamma=5.0)
    p2 = models.electromag2_blocks(n=64, cpml=10, nt=200, src=(32, 12), nrec=16, rec_z=6, nblocks=5)
    p2.model["e13"][:] = 0.4
    p2.model["s13"][:] = 2e-4
    p3 = models.seismic25_two_layer(n=48, cpml=8, nt=120, nrec=12)
    p4 = models.electromag25_blocks(n=48, cpml=8, nt=150, nrec=12)
    p5 = models.seismic3_layers(n=24, cpml=6, nt=40, nlayers=3, nrec_side=4, rec_z=3, src_z=6)
    p6 = models.electromag3_blocks(n=22, cpml=5, nt=60, nblocks=4, nrec_side=4, f0=8e8)
    for c in ("s12", "s13", "s23"):  # full conductivity tensor: every coupling term
        p6.model[c][:] = 1e-3
    return {"seismic2": p1, "electromag2": p2, "seismic25": p3, "electromag25": p4, "seismic3": p5,
            "electromag3": p6}


PROBLEMS = small_problems()


@pytest.mark.parametrize("name", list(PROBLEMS))
def test_fp64_bit_exact(oracle, name):
    p = PROBLEMS[name]
    o = oracle.run_oracle(p)
    g = sg.run(p, sg.FP64)
    assert_exact(g, o)


@pytest.mark.parametrize("name", list(PROBLEMS))
def test_fp32_rel_l2(oracle, name):
    p = PROBLEMS[name]
    o = oracle.run_oracle(p)
    g = sg.run(p, sg.FP32)
    assert rel_l2(g["traces"], o["traces"]) <= FP32_TOL
    for q in range(len(o["fields"])):
        if np.linalg.norm(o["fields"][q]) > 0:
            assert rel_l2(g["fields"][q], o["fields"][q]) <= FP32_TOL, f"field {q}"


@pytest.mark.parametrize("density", ["harmonic", "geometric", "arithmetic", "none"])
def test_seismic2_density_and_stress_source(oracle, density):
    p = models.seismic2_two_layer(n=48, cpml=8, nt=100, src=(24, 10), nrec=8, rec_z=4, density=density, gamma=3.0)
    p.src["xx"] = 0.2 * p.src["z"]
    p.src["xz"] = -0.3 * p.src["z"]
    p.src["zz"] = 0.1 * p.src["z"]
    assert_exact(sg.run(p, sg.FP64), oracle.run_oracle(p))


def test_seismic3_stress_source_and_norms(oracle):
    p = models.seismic3_layers(n=20, cpml=5, nt=30, nlayers=2, nrec_side=3, rec_z=2, src_z=5, density="harmonic")
    for k in ("xx", "xy", "xz", "yy", "yz", "zz"):
        p.src[k] = 0.05 * p.src["z"]
    p.src["x"] = 0.5 * p.src["z"]
    p.src["y"] = -0.5 * p.src["z"]
    assert_exact(sg.run(p, sg.FP64), oracle.run_oracle(p))


@pytest.mark.parametrize("density", ["harmonic", "geometric", "arithmetic", "none"])
def test_seismic3_fp32_stress_source_density(oracle, density):
    """FP32 z-marching kernels: every source term, density rule and norm."""
    p = models.seismic3_layers(n=30, cpml=6, nt=40, nlayers=3, nrec_side=4, rec_z=3, src_z=7, density=density)
    for k in ("xx", "xy", "xz", "yy", "yz", "zz"):
        p.src[k] = 0.05 * p.src["z"]
    p.src["x"] = 0.5 * p.src["z"]
    p.src["y"] = -0.5 * p.src["z"]
    o = oracle.run_oracle(p)
    g = sg.run(p, sg.FP32)
    assert rel_l2(g["traces"], o["traces"]) <= FP32_TOL
    for q in range(9):
        assert rel_l2(g["fields"][q], o["fields"][q]) <= FP32_TOL, f"field {q}"
    assert rel_l2(g["norms"], o["norms"]) <= FP32_TOL
    for q in range(45):
        if np.linalg.norm(o["memory"][q]) > 0:
            assert rel_l2(g["memory"][q], o["memory"][q]) <= 10 * FP32_TOL, f"memory {q}"


@pytest.mark.parametrize("name", ["seismic2", "electromag2", "seismic3", "electromag3"])
def test_chunked_stepping_matches_one_shot(name):
    """Graph chunks of different lengths (and a tail) give the same state."""
    p = PROBLEMS[name]
    ref = sg.run(p, sg.FP64)
    with sg.Solver(p, sg.FP64) as s:
        for n in (1, 7, 64, 13):
            if s.steps_done + n <= p.time_steps:
                s.step(n)
        s.step(p.time_steps - s.steps_done)
        s.sync()
        tr, nrm = s.traces()
        f = s.get_fields()
    assert np.array_equal(tr, ref["traces"])
    for a, b in zip(f, ref["fields"]):
        assert np.array_equal(a, b)


def test_no_cpml_and_no_receivers(oracle):
    """cpml = 0 (empty PML) and zero receivers."""
    p = models.seismic2_two_layer(n=32, cpml=0, nt=40, src=(16, 10), nrec=4, rec_z=4)
    p.receivers = None
    g = sg.run(p, sg.FP64)
    o = oracle.run_oracle(p)
    for a, b in zip(g["fields"], o["fields"]):
        assert np.array_equal(a, b)
    assert np.array_equal(g["norms"], o["norms"])


def test_source_on_edge_is_zeroed(oracle):
    """A source on the Dirichlet ring is injected and then zeroed, as in the reference."""
    p = models.seismic2_two_layer(n=24, cpml=4, nt=30, src=(-3, 10), nrec=4, rec_z=4)
    assert p.source_cell() % p.nx == 0
    assert_exact(sg.run(p, sg.FP64), oracle.run_oracle(p))


def test_unstable_reports_error(oracle):
    """dt far above the CFL limit blows up; the solver returns SEIDART_ERR_UNSTABLE."""
    p = models.seismic2_two_layer(n=32, cpml=4, nt=400, src=(16, 10), nrec=4, rec_z=4)
    p.dt *= 4.0
    o = oracle.run_oracle(p)
    assert o["blowup"] is not None
    with pytest.raises(sg.UnstableError) as e:
        sg.run(p, sg.FP64)
    assert f"step {o['blowup']}" in str(e.value)


def test_electromag3_initial_fields_and_interior_box(oracle):
    """electromag3 from nonzero initial E (initialconditionEx/Ey/Ez) on a grid
    whose interior holds an inert box (cells that skip the C-PML memories),
    FP64 bit-exact, including the H faces that are zeroed on read-back."""
    p = models.electromag3_blocks(n=36, cpml=6, nt=25, nblocks=3, nrec_side=3, f0=8e8)
    rng = np.random.default_rng(11)
    for q, nm in enumerate(("Ex", "Ey", "Ez")):
        p.fields0[nm] = np.asfortranarray(rng.normal(0, 1e-3, p.shape))
    assert_exact(sg.run(p, sg.FP64), oracle.run_oracle(p))


def test_seismic3_fp32_velocity_pair_kernel(oracle, monkeypatch):
    """The cell-pair velocity kernel (two x-adjacent cells per thread, float2
    loads on lean tiles) against the one-cell kernel and the oracle, on a grid
    with lean tiles, a source inside and an odd tile tail in y."""
    p = models.seismic3_layers(n=72, cpml=8, nt=30, nlayers=3, nrec_side=4, rec_z=3, src_z=30, ny=58)
    p.src["x"] = 0.5 * p.src["z"]
    out = {}
    for flag in ("0", "1"):
        monkeypatch.setenv("SEIDART_S3_VPAIR", flag)
        out[flag] = sg.run(p, sg.FP32)
    for a, b in zip(out["0"]["fields"], out["1"]["fields"]):
        assert rel_l2(b, a) <= 1e-6
    assert rel_l2(out["1"]["norms"], out["0"]["norms"]) <= 1e-6
    o = oracle.run_oracle(p)
    for q in range(9):
        assert rel_l2(out["1"]["fields"][q], o["fields"][q]) <= FP32_TOL, q


def test_seismic3_fp32_velocity_warp_parts(oracle, monkeypatch):
    """The pair velocity kernel's lean test per warp (32 x 2 cells) against
    one test per 32 x 16 tile, on a grid with a ragged y tail, a force and a
    stress source and C-PML faces that cut through tiles: more cells take the
    lean path, whose expressions are the one-cell path's (within 1e-6, as the
    one-cell kernel), and the result stays within FP32_TOL of the oracle."""
    p = models.seismic3_layers(n=84, cpml=10, nt=40, nlayers=3, nrec_side=4, rec_z=3, src_z=12, ny=70)
    p.src["x"] = 0.5 * p.src["z"]
    p.src["xx"] = 1e6 * p.src["z"]
    out = {}
    for flag in ("0", "1"):
        monkeypatch.setenv("SEIDART_S3_VSUB", flag)
        with sg.Solver(p, sg.FP32) as s:
            s.step(p.time_steps)
            s.sync()
            tr, nrm = s.traces()
            out[flag] = (s.get_fields(), s.get_memory(), tr, nrm)
    a, b = out["0"], out["1"]
    assert np.max(np.abs(a[2])) > 0 and max(np.max(np.abs(a[1][q])) for q in range(36, 45)) > 0
    errs = {"traces": rel_l2(b[2], a[2]), "norms": rel_l2(b[3], a[3])}
    for q in range(9):
        errs[f"field {q}"] = rel_l2(b[0][q], a[0][q])
    for q in range(36, 45):
        errs[f"memory {q}"] = rel_l2(b[1][q], a[1][q])
    print({k: float(v) for k, v in errs.items()})
    assert max(errs.values()) <= 1e-6, errs
    o = oracle.run_oracle(p)
    assert rel_l2(b[2], o["traces"]) <= FP32_TOL
    for q in range(9):
        assert rel_l2(b[0][q], o["fields"][q]) <= FP32_TOL, q


def test_seismic3_fp32_odd_sizes(oracle):
    """Odd nx and ny: the staged stress and the cell-pair velocity kernels
    need nx % 4 == 0 and nx even, so the bulk-copy stress and the one-cell
    velocity kernels run (ragged last tiles in x and y)."""
    p = models.seismic3_layers(n=35, cpml=5, nt=30, nlayers=2, nrec_side=3, rec_z=3, src_z=6, ny=29)
    assert p.nx % 2 == 1 and p.ny % 2 == 1
    o = oracle.run_oracle(p)
    g = sg.run(p, sg.FP32)
    for q in range(9):
        assert rel_l2(g["fields"][q], o["fields"][q]) <= FP32_TOL, q
    assert rel_l2(g["norms"], o["norms"]) <= FP32_TOL


@pytest.mark.parametrize("name", ["seismic2", "electromag3"])
def test_zero_steps_is_a_clean_error(name):
    """time_steps = 0 is refused with SEIDART_ERR_ARG (the reference would
    loop zero times); the context stays usable."""
    from dataclasses import replace
    p = replace(PROBLEMS[name], time_steps=0, src={})
    with pytest.raises(sg.SeidartError, match="time_steps"):
        sg.run(p, sg.FP64)
    g = sg.run(replace(PROBLEMS[name], time_steps=2, src={}), sg.FP64)
    assert g["traces"].shape[0] == 2


def test_electromag3_no_cpml_source_on_face(oracle):
    """electromag3 with cpml = 0 (no PML; every cell inside the box) and the
    source on a Dirichlet face: injected, then zeroed, as in the reference."""
    p = models.electromag3_blocks(n=14, cpml=0, nt=20, nblocks=2, nrec_side=2, f0=8e8)
    p.xind = 1  # source cell x = 1 (1-based): the low-x face
    assert_exact(sg.run(p, sg.FP64), oracle.run_oracle(p))
