"""The host thread pool behind the solver's set-up and transfer loops
(csrc/host_pool.h), compiled with g++ and exercised on the CPU."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_host_pool_ranges_concurrency_and_fork(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = tmp_path / "host_pool_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", str(ROOT / "seidart-backend_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "host_pool_check.cc"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok"), out.stdout
