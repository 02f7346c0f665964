"""Plane-wave sources (csrc/planewave.cu; plane_wave_source.f08 and the
plane-wave branches of cpmlfdtd.f08).

CPU: the host set-up (Jacobi eigenvalues of the Mandel stiffness or the
permittivity over the distinct material tuples) gives the background speed
and impedance that LAPACK gives the oracle; the propagation direction and
polarisation follow rotmat with Fortran's column-filling reshape; the
injection faces are the ones p points into.
GPU: every family with a plane wave against the oracle -- FP64 within 1e-12
relative L2 (the wavelet's exp is CUDA's on the device and the C library's
in the oracle, so not bit for bit), FP32 within 1e-4 -- and the file
contract with source_type "pwp" / "pw".
"""
import ctypes as C
import os
import subprocess
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

import seidart_gpu as sg
from seidart_gpu import _lib, models

FP64_TOL = 1e-12
FP32_TOL = 1e-4

pytestmark_lib = pytest.mark.skipif(not _lib.LIB_PATH.exists(), reason="library not built")


def _setup(problem, pw):
    L = C.CDLL(str(_lib.LIB_PATH))
    L.seidart_plane_wave_setup.restype = C.c_int
    L.seidart_plane_wave_setup.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    out = np.zeros(15)
    model = problem.model_list()
    arr = _lib.ptr_array(model)
    p = replace(problem, plane_wave=pw)
    rc = L.seidart_plane_wave_setup(problem.family, C.byref(problem.domain()), C.byref(problem.source()),
                                    C.byref(p.plane_wave_struct()), arr, out.ctypes.data)
    assert rc == 0
    return out


def _fortran_direction(xz, xy, yz):
    """rotmat / direction_polarization_vector with Fortran's reshape (columns)."""
    d = np.pi / 180.0
    cx, cy, cz = np.cos(d * yz), np.cos(d * xz), np.cos(d * xy)
    sx, sy, sz = np.sin(d * yz), np.sin(d * xz), np.sin(d * xy)
    Rx = np.reshape([1, 0, 0, 0, cx, -sx, 0, sx, cx], (3, 3), order="F")
    Ry = np.reshape([cy, 0, sy, 0, 1, 0, -sy, 0, cy], (3, 3), order="F")
    Rz = np.reshape([cz, -sz, 0, sz, cz, 0, 0, 0, 1], (3, 3), order="F")
    R = Ry @ (Rz @ Rx)
    p = R @ np.array([0.0, 0.0, 1.0])
    p = p / np.linalg.norm(p)
    t = R @ np.array([1.0, 0.0, 0.0])
    t = t - np.dot(t, p) * p
    return p, t / np.linalg.norm(t)


def _aniso2d(seed=3):
    p = models.seismic2_two_layer(n=32, cpml=6, nt=60, src=(16, 8), nrec=6, rec_z=4)
    rng = np.random.default_rng(seed)
    for k in ("c15", "c35"):
        p.model[k] = np.asfortranarray(p.model[k] + rng.uniform(-1e8, 1e8) * np.ones(p.shape))
    return p


# ------------------------------------------------------------------- CPU
@pytestmark_lib
@pytest.mark.parametrize("angles", [(0.0, 0.0, 0.0), (30.0, 0.0, 0.0), (-40.0, 0.0, 0.0), (25.0, 35.0, 10.0),
                                    (120.0, -20.0, 5.0)])
def test_direction_follows_rotmat(angles):
    p0 = models.seismic3_layers(n=12, cpml=3, nt=5, nlayers=2, nrec_side=2, rec_z=2, src_z=4)
    out = _setup(p0, {"kind": "pw", "frequency": 50.0, "x_z_rotation": angles[0], "x_y_rotation": angles[1],
                      "y_z_rotation": angles[2]})
    p, e = _fortran_direction(*angles)
    assert np.allclose(out[2:5], p, atol=1e-15) and np.allclose(out[5:8], e, atol=1e-15)
    want = [ax for ax in range(3) if abs(p[ax]) > 1e-6]
    assert int(out[8]) == len(want) and list(out[9:9 + len(want)].astype(int)) == want
    for f, ax in enumerate(want):  # XMIN face when p points in, XMAX when it points out
        n = (p0.nx, p0.ny, p0.nz)[ax]
        assert int(out[12 + f]) == (p0.cpml if p[ax] > 0 else n - p0.cpml - 1)


@pytestmark_lib
def test_background_speed_matches_lapack(oracle):
    cases = [(_aniso2d(), {"kind": "pw"}),
             (models.seismic3_layers(n=12, cpml=3, nt=5, nlayers=3, nrec_side=2, rec_z=2, src_z=4), {"kind": "pwp"}),
             (models.seismic25_two_layer(n=16, cpml=4, nt=5, nrec=2), {"kind": "pw"}),
             (models.electromag2_blocks(n=24, cpml=4, nt=5, src=(12, 6), nrec=2, rec_z=3, nblocks=4), {"kind": "pw"}),
             (models.electromag3_blocks(n=12, cpml=3, nt=5, nblocks=3, nrec_side=2), {"kind": "pw"})]
    cases[3][0].model["e13"][:] = 0.7
    for prob, pw in cases:
        pw = dict(pw, frequency=1.0e3, x_z_rotation=20.0)
        out = _setup(prob, pw)
        v, eta = oracle.plane_wave_background(replace(prob, plane_wave=pw))
        assert abs(out[0] - v) <= 1e-13 * v, (prob.family, out[0], v)
        if eta:
            assert abs(out[1] - eta) <= 1e-13 * eta


# ------------------------------------------------------------------- GPU
def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


def _pw_cases():
    s2 = _aniso2d()
    s2 = replace(s2, time_steps=70, src={}, plane_wave={"kind": "pw", "wavelet": "gaus1", "frequency": 600.0,
                                                        "x_z_rotation": 30.0, "amplitude": 2.0})
    s2p = replace(s2, plane_wave={"kind": "pwp", "wavelet": "gaus2", "frequency": 600.0, "x_z_rotation": -25.0})
    s25 = models.seismic25_two_layer(n=32, cpml=6, nt=60, nrec=6)
    s25 = replace(s25, src={}, plane_wave={"kind": "pw", "wavelet": "gaus1", "frequency": 600.0,
                                           "x_z_rotation": 35.0})
    s3 = models.seismic3_layers(n=20, cpml=4, nt=40, nlayers=2, nrec_side=3, rec_z=3, src_z=5)
    s3 = replace(s3, src={}, plane_wave={"kind": "pw", "wavelet": "gaus1", "frequency": 1500.0,
                                         "x_z_rotation": 30.0, "x_y_rotation": 40.0, "y_z_rotation": 15.0})
    # 104^3 cells: the FP32 fast kernels' lean tiles exist, and the
    # injection faces cross some of them
    s3l = models.seismic3_layers(n=88, cpml=8, nt=40, nlayers=3, nrec_side=4, rec_z=3, src_z=10)
    s3l = replace(s3l, src={}, plane_wave={"kind": "pw", "wavelet": "gaus1", "frequency": 400.0,
                                           "x_z_rotation": 25.0, "x_y_rotation": 35.0, "y_z_rotation": 10.0})
    e2 = models.electromag2_blocks(n=40, cpml=6, nt=80, src=(20, 8), nrec=6, rec_z=5, nblocks=3)
    e2.model["e13"][:] = 0.5
    e2 = replace(e2, src={}, plane_wave={"kind": "pw", "wavelet": "gaus1", "frequency": 1.0e9,
                                         "x_z_rotation": 20.0})
    e3 = models.electromag3_blocks(n=20, cpml=4, nt=50, nblocks=2, nrec_side=3)
    e3 = replace(e3, src={}, plane_wave={"kind": "pw", "wavelet": "gaus0", "frequency": 1.5e9,
                                         "x_z_rotation": -30.0, "x_y_rotation": 20.0, "y_z_rotation": 25.0})
    return {"seismic2": s2, "seismic2_p": s2p, "seismic25": s25, "seismic3": s3, "seismic3_lean": s3l,
            "electromag2": e2, "electromag3": e3}


PW = _pw_cases() if _lib.LIB_PATH.exists() else {}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(PW) or ["none"])
def test_plane_wave_fp64_matches_oracle(oracle, name):
    p = PW[name]
    o = oracle.run_oracle(p)
    g = sg.run(p, sg.FP64)
    assert np.max(np.abs(o["traces"])) > 0
    assert _rel(g["traces"], o["traces"]) <= FP64_TOL
    for q, (a, b) in enumerate(zip(g["fields"], o["fields"])):
        assert _rel(a, b) <= FP64_TOL, f"field {q}: {_rel(a, b)}"
    assert _rel(g["norms"], o["norms"]) <= FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(PW) or ["none"])
def test_plane_wave_fp32(oracle, name):
    p = PW[name]
    o = oracle.run_oracle(p)
    g = sg.run(p, sg.FP32)
    assert _rel(g["traces"], o["traces"]) <= FP32_TOL
    assert _rel(g["norms"], o["norms"]) <= FP32_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["seismic2_p", "electromag2"])
def test_plane_wave_file_contract(tmp_path, oracle, name):
    from seidart_gpu import fortran_io as fio
    p = PW[name]
    seismic = p.family == sg.SEISMIC2
    fio.write_problem(p, tmp_path)
    pkg = Path(sg.__file__).resolve().parent
    r = subprocess.run([str(pkg / "seidartfdtd"), "input.json", f"seismic={'true' if seismic else 'false'}"],
                       cwd=tmp_path, capture_output=True, text=True, env=dict(os.environ))
    assert r.returncode == 0, r.stderr + r.stdout
    o = oracle.run_oracle(p)
    ch = "Vz" if seismic else "Ez"
    snap = fio.read_record(tmp_path / fio.snapshot_name(ch, p.time_steps, p.xind, p.zind), np.float32, p.shape)
    want = o["fields"][1].astype(np.float32)
    assert np.max(np.abs(want)) > 0
    assert np.max(np.abs(snap - want)) <= 1e-6 * np.max(np.abs(want))
