"""The reference's file contract end to end on the GPU: .dat inputs written
the way the frontend writes them, the `seidartfdtd` driver (and the legacy
C entry points through the Python module), per-step float32 snapshots
compared with the CPU restatement."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import fortran_io as fio
from seidart_gpu import models

pytestmark = pytest.mark.gpu
PKG = Path(sg.__file__).resolve().parent


def _snap(d, chan, it, p, threeD=False):
    name = fio.snapshot_name(chan, it, p.xind, p.zind, p.yind if threeD else None)
    return fio.read_record(d / name, np.float32, p.shape)


@pytest.mark.parametrize("family", ["seismic2", "electromag2"])
def test_cli_snapshots_match_oracle(tmp_path, oracle, family):
    if family == "seismic2":
        p = models.seismic2_two_layer(n=40, cpml=6, nt=25, src=(20, 8), nrec=4, rec_z=4)
        args, chans = ["seismic=true"], ("Vx", "Vz")
    else:
        p = models.electromag2_blocks(n=40, cpml=6, nt=25, src=(20, 8), nrec=4, rec_z=4, nblocks=3)
        args, chans = ["seismic=false"], ("Ex", "Ez")
    fio.write_problem(p, tmp_path)
    r = subprocess.run([str(PKG / "seidartfdtd"), "input.json", *args], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for it in (1, 13, 25):
        o = oracle.run_oracle(p, nsteps=it)
        for q, ch in enumerate(chans):
            snap = _snap(tmp_path, ch, it, p)
            assert np.array_equal(snap, o["fields"][q].astype(np.float32)), f"{ch} step {it}"
    assert len(list(tmp_path.glob(f"{chans[0]}.*.dat"))) == p.time_steps


def test_cli_seismic3_norm_files(tmp_path, oracle):
    p = models.seismic3_layers(n=12, cpml=4, nt=8, nlayers=2, nrec_side=2, rec_z=2, src_z=4)
    fio.write_problem(p, tmp_path)
    r = subprocess.run([sys.executable, "-m", "seidart_gpu.cli", "input.json", "seismic=true"], cwd=tmp_path,
                       capture_output=True, text=True, env={**os.environ, "PYTHONPATH": str(PKG.parent)})
    assert r.returncode == 0, r.stderr + r.stdout
    o = oracle.run_oracle(p)
    assert np.array_equal(_snap(tmp_path, "Vz", 8, p, threeD=True), o["fields"][2].astype(np.float32))
    vn = fio.read_record(tmp_path / "velocity_norm.dat")
    sn = fio.read_record(tmp_path / "stress_norm.dat")
    assert np.array_equal(vn, o["norms"][0]) and np.array_equal(sn, o["norms"][1])


def test_cli_electromag3_snapshots(tmp_path, oracle):
    """dim = 3 with seismic=false runs electromag3 (main.f08:88-97): 3D Ex/Ey/Ez snapshots."""
    p = models.electromag3_blocks(n=12, cpml=4, nt=10, nblocks=2, nrec_side=2, f0=8e8)
    fio.write_problem(p, tmp_path)
    r = subprocess.run([str(PKG / "seidartfdtd"), "input.json", "seismic=false"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "3D electromagnetic" in r.stdout
    for it in (1, 10):
        o = oracle.run_oracle(p, nsteps=it)
        for q, ch in enumerate(("Ex", "Ey", "Ez")):
            snap = _snap(tmp_path, ch, it, p, threeD=True)
            assert np.array_equal(snap, o["fields"][q].astype(np.float32)), f"{ch} step {it}"
    assert not (tmp_path / "velocity_norm.dat").exists()


@pytest.mark.parametrize("family", ["seismic25", "electromag25"])
def test_cli_25d_zstd_blocks(tmp_path, oracle, family):
    """2.5D default output: zstd blocks of FDTD_STEPS_PER_BLOCK steps, float32
    real parts with the CPML stripped, (x, 1, z, component, step)."""
    if family == "seismic25":
        p = models.seismic25_two_layer(n=20, cpml=5, nt=17, nrec=4)
        args, prefix = ["seismic=true"], "S25"
    else:
        p = models.electromag25_blocks(n=20, cpml=5, nt=17, nrec=4)
        args, prefix = ["seismic=false"], "EM25"
    fio.write_problem(p, tmp_path)
    env = {**os.environ, "FDTD_STEPS_PER_BLOCK": "7", "KY": repr(p.ky), "DENSITY_METHOD": p.density}
    env.pop("FDTD_LEGACY_OUTPUT", None)
    r = subprocess.run([str(PKG / "seidartfdtd"), "input.json", *args], cwd=tmp_path, capture_output=True,
                       text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert not list(tmp_path.glob("V*.dat")) and not list(tmp_path.glob("E[xyz].*.dat"))
    c, onx, onz = p.cpml, p.nx - 2 * p.cpml, p.nz - 2 * p.cpml
    st = oracle.OracleState(p)
    for first, last in ((1, 7), (8, 14), (15, 17)):
        name = fio.block_name(prefix, first, last, p.xind, p.yind, p.zind)
        blk = fio.read_block(tmp_path / name, onx, onz)
        assert blk.shape == (onx, 1, onz, 3, last - first + 1)
        for it in range(first, last + 1):
            st.step(1)
            for q in range(3):
                want = np.real(st.fields[q][c:c + onx, c:c + onz]).astype(np.float32)
                assert np.array_equal(blk[:, 0, :, q, it - first], want), (name, it, q)
    assert len(list(tmp_path.glob("*.blk.zst"))) == 3


def test_cli_25d_legacy_output(tmp_path):
    """FDTD_LEGACY_OUTPUT=TRUE: per-step Vx/Vy/Vz files, no blocks."""
    p = models.seismic25_two_layer(n=16, cpml=4, nt=5, nrec=4)
    fio.write_problem(p, tmp_path)
    env = {**os.environ, "FDTD_LEGACY_OUTPUT": "TRUE"}
    r = subprocess.run([str(PKG / "seidartfdtd"), "input.json", "seismic=true"], cwd=tmp_path,
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert not list(tmp_path.glob("*.blk.zst"))
    assert len(list(tmp_path.glob("Vy.*.dat"))) == p.time_steps


def test_legacy_entry_point(tmp_path, oracle, monkeypatch):
    """cpmlfdtd.seismic2(nx, nz, dx, dz, src, npml, nstep) with the legacy dt rule."""
    from seidart_gpu import cpmlfdtd
    p = models.seismic2_two_layer(n=32, cpml=5, nt=20, src=(16, 6), nrec=4, rec_z=4)
    m = p.model
    p.dt = min(p.dx, p.dz) / np.sqrt(3.0 * max(np.max(m["c11"] / m["rho"]), np.max(m["c33"] / m["rho"])))
    p.src["z"] = models.ricker(p.time_steps, p.dt, 60.0)
    fio.write_problem(p, tmp_path)
    monkeypatch.chdir(tmp_path)
    cpmlfdtd.seismic2(p.nx, p.nz, p.dx, p.dz, np.array([p.xind, p.zind]), p.cpml, p.time_steps)
    o = oracle.run_oracle(p)
    assert np.array_equal(_snap(tmp_path, "Vz", p.time_steps, p), o["fields"][1].astype(np.float32))


def test_legacy_3d_entry_points(tmp_path, oracle, monkeypatch):
    """cpmlfdtd.seismic25 / electromag25 (the binding's 3D solvers) write 3D
    snapshots of the 3D loops, dt from the legacy 3D rules."""
    from seidart_gpu import cpmlfdtd
    monkeypatch.chdir(tmp_path)
    p = models.seismic3_layers(n=10, cpml=3, nt=6, nlayers=2, nrec_side=2, rec_z=2, src_z=4)
    m = p.model
    h = min(p.dx, p.dy, p.dz)
    p.dt = 0.7 * h / np.sqrt(3.0 * max(np.max(m["c11"] / m["rho"]), np.max(m["c22"] / m["rho"]),
                                       np.max(m["c33"] / m["rho"])))
    fio.write_problem(p, tmp_path)
    cpmlfdtd.seismic25(p.nx, p.ny, p.nz, p.dx, p.dy, p.dz, np.array([p.xind, p.yind, p.zind]), p.cpml,
                       p.time_steps)
    o = oracle.run_oracle(p)
    assert np.array_equal(_snap(tmp_path, "Vz", p.time_steps, p, threeD=True), o["fields"][2].astype(np.float32))
    q = models.electromag3_blocks(n=10, cpml=3, nt=6, nblocks=1, nrec_side=2, f0=8e8)
    emin = min(np.min(q.model[k]) for k in ("e11", "e22", "e33"))
    q.dt = min(q.dx, q.dy, q.dz) / (2.0 * 2.9979458e8 / np.sqrt(emin))
    fio.write_problem(q, tmp_path)
    cpmlfdtd.electromag25(q.nx, q.ny, q.nz, q.dx, q.dy, q.dz, np.array([q.xind, q.yind, q.zind]), q.cpml,
                          q.time_steps)
    o = oracle.run_oracle(q)
    assert np.array_equal(_snap(tmp_path, "Ez", q.time_steps, q, threeD=True), o["fields"][2].astype(np.float32))


def test_missing_input_is_an_error(tmp_path):
    p = models.seismic2_two_layer(n=24, cpml=4, nt=5, src=(12, 6), nrec=2, rec_z=3)
    fio.write_problem(p, tmp_path)
    (tmp_path / "c33.dat").unlink()
    r = subprocess.run([str(PKG / "seidartfdtd"), "input.json"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "c33.dat" in r.stderr
