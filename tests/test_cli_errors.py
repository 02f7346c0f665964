"""The seidartfdtd program's input checks, made before any device work, so
they run without a GPU: a missing or malformed input.json, a missing `.dat`
record and a record of the wrong size each stop the run with a message
naming the file and a non-zero exit status (the reference stops with a
message too, seidartio.f08), and valid input on a host without a GPU is
refused rather than run on a CPU fallback."""
import pathlib
import subprocess

import pytest
import torch

from seidart_gpu import fortran_io as fio
from seidart_gpu import models

ROOT = pathlib.Path(__file__).resolve().parents[1]
EXE = ROOT / "seidart-backend_gb300" / "seidart_gpu" / "seidartfdtd"


def _run(cwd, *args):
    if not EXE.exists():
        pytest.skip("seidartfdtd is not built")
    return subprocess.run([str(EXE), *args], cwd=cwd, capture_output=True, text=True, timeout=120)


def _write(tmp_path):
    p = models.seismic2_two_layer(n=24, cpml=4, nt=5, src=(12, 6), nrec=2, rec_z=3)
    fio.write_problem(p, tmp_path)
    return p


def test_missing_input_json(tmp_path):
    r = _run(tmp_path, "input.json")
    assert r.returncode != 0 and "input.json" in r.stderr


def test_malformed_input_json(tmp_path):
    (tmp_path / "input.json").write_text('{"Domain": ')
    r = _run(tmp_path, "input.json")
    assert r.returncode != 0 and "malformed JSON" in r.stderr


def test_missing_record(tmp_path):
    _write(tmp_path)
    (tmp_path / "c33.dat").unlink()
    r = _run(tmp_path, "input.json")
    assert r.returncode != 0 and "c33.dat" in r.stderr


def test_record_of_the_wrong_size(tmp_path):
    _write(tmp_path)
    data = (tmp_path / "rho.dat").read_bytes()
    (tmp_path / "rho.dat").write_bytes(data[:len(data) // 2])
    r = _run(tmp_path, "input.json")
    assert r.returncode != 0 and "rho.dat" in r.stderr


def test_valid_input_without_a_gpu_is_refused(tmp_path):
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    _write(tmp_path)
    r = _run(tmp_path, "input.json")
    assert r.returncode != 0 and "no CUDA device" in r.stderr
