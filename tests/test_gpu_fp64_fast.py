"""Fast FP64 solvers (SEIDART_FP64_FAST) against the CPU restatement.

FP64 fields with the fast path's arithmetic: reciprocals set up on the host
(1/kappa, 1/(1 + gamma dt), 1/dx, buoyancies) instead of the reference's
divisions, and FMA contraction.  Not bit-identical to the reference's
operation order; every field, CPML memory array, receiver trace and
max-norm must stay within FP64_FAST_TOL relative L2 of the oracle, on the
small cases of every family and on full-length 2D runs.
"""
import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import models

from test_gpu_parity import PROBLEMS
from test_plane_wave import PW

pytestmark = pytest.mark.gpu

FP64_FAST_TOL = 1e-12  # relative L2 against the FP64 oracle


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


def assert_close(g, o, tol=FP64_FAST_TOL, memory=True):
    assert np.max(np.abs(o["traces"])) > 0
    assert rel_l2(g["traces"], o["traces"]) <= tol, rel_l2(g["traces"], o["traces"])
    for q, (a, b) in enumerate(zip(g["fields"], o["fields"])):
        assert rel_l2(a, b) <= tol, f"field {q}: {rel_l2(a, b)}"
    assert rel_l2(g["norms"], o["norms"]) <= tol
    if memory:
        for q, (a, b) in enumerate(zip(g["memory"], o["memory"])):
            if np.linalg.norm(b) > 0:
                assert rel_l2(a, b) <= tol, f"memory {q}: {rel_l2(a, b)}"


@pytest.mark.parametrize("name", list(PROBLEMS))
def test_fp64_fast_matches_oracle(oracle, name):
    p = PROBLEMS[name]
    o = oracle.run_oracle(p)
    g = sg.run(p, sg.FP64_FAST)
    assert_close(g, o)
    # it is the fast arithmetic, not the exact build under another name
    e = sg.run(p, sg.FP64)
    assert any(not np.array_equal(a, b) for a, b in zip(g["fields"], e["fields"]))


@pytest.mark.parametrize("density", ["harmonic", "geometric", "arithmetic", "none"])
def test_fp64_fast_density_rules_and_stress_sources(oracle, density):
    p = models.seismic2_two_layer(n=48, cpml=8, nt=100, src=(24, 10), nrec=8, rec_z=4, density=density, gamma=3.0)
    p.src["xx"] = 0.2 * p.src["z"]
    p.src["xz"] = -0.3 * p.src["z"]
    p.src["zz"] = 0.1 * p.src["z"]
    assert_close(sg.run(p, sg.FP64_FAST), oracle.run_oracle(p))
    p3 = models.seismic3_layers(n=20, cpml=5, nt=30, nlayers=2, nrec_side=3, rec_z=2, src_z=5, density=density)
    for k in ("xx", "xy", "xz", "yy", "yz", "zz"):
        p3.src[k] = 0.05 * p3.src["z"]
    p3.src["x"] = 0.5 * p3.src["z"]
    p3.src["y"] = -0.5 * p3.src["z"]
    assert_close(sg.run(p3, sg.FP64_FAST), oracle.run_oracle(p3))


def test_fp64_fast_full_length_2d(oracle):
    """The 256^2 + 20 CPML two-layer run for all 2000 steps, and a 256^2 GPR
    run for 4000 steps: rounding differences do not grow past the bound.
    The GPR field has left the grid or decayed in the conductive blocks long
    before step 4000, so its final snapshot is held against the norm of the
    snapshot at step 1500, when the wave fills the grid (relative to its own
    small norm, the late residual differs by a few 1e-12)."""
    p = models.seismic2_two_layer()
    assert_close(sg.run(p, sg.FP64_FAST), oracle.run_oracle(p), memory=False)
    e = models.electromag2_blocks(n=256, nt=4000, src=(128, 30), nrec=32, rec_z=25, nblocks=6)
    st = oracle.OracleState(e)
    with sg.Solver(e, sg.FP64_FAST) as s:
        s.step(1500)
        st.step(1500)
        mid = [f.copy() for f in st.fields]
        for q, (a, b) in enumerate(zip(s.get_fields(), mid)):
            assert rel_l2(a, b) <= FP64_FAST_TOL, f"step 1500 field {q}: {rel_l2(a, b)}"
        s.step(2500)
        st.step(2500)
        tr, nrm = s.traces()
        o = st.result()
        assert rel_l2(tr, o["traces"]) <= FP64_FAST_TOL
        assert rel_l2(nrm, o["norms"]) <= FP64_FAST_TOL
        for q, (a, b) in enumerate(zip(s.get_fields(), o["fields"])):
            err = np.linalg.norm((a - b).ravel()) / np.linalg.norm(mid[q].ravel())
            assert err <= FP64_FAST_TOL, f"step 4000 field {q}: {err}"


@pytest.mark.parametrize("name", list(PW) or ["none"])
def test_fp64_fast_plane_waves(oracle, name):
    p = PW[name]
    assert_close(sg.run(p, sg.FP64_FAST), oracle.run_oracle(p), memory=False)


def test_cli_precision_fp64fast(tmp_path, oracle):
    """`seidartfdtd input.json precision=fp64fast`: the file contract on the
    fast FP64 solver; float32 snapshots agree with the oracle's to float32
    rounding."""
    import subprocess
    from pathlib import Path
    from seidart_gpu import fortran_io as fio
    p = models.electromag2_blocks(n=40, cpml=6, nt=25, src=(20, 8), nrec=4, rec_z=4, nblocks=3)
    fio.write_problem(p, tmp_path)
    exe = Path(sg.__file__).resolve().parent / "seidartfdtd"
    r = subprocess.run([str(exe), "input.json", "seismic=false", "precision=fp64fast"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    o = oracle.run_oracle(p)
    for q, ch in enumerate(("Ex", "Ez")):
        snap = fio.read_record(tmp_path / fio.snapshot_name(ch, p.time_steps, p.xind, p.zind), np.float32, p.shape)
        want = o["fields"][q].astype(np.float32)
        assert np.max(np.abs(want)) > 0
        assert np.max(np.abs(snap - want)) <= 1e-6 * np.max(np.abs(want)), ch
