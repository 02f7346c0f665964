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


def test_missing_input_is_an_error(tmp_path):
    p = models.seismic2_two_layer(n=24, cpml=4, nt=5, src=(12, 6), nrec=2, rec_z=3)
    fio.write_problem(p, tmp_path)
    (tmp_path / "c33.dat").unlink()
    r = subprocess.run([str(PKG / "seidartfdtd"), "input.json"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "c33.dat" in r.stderr
