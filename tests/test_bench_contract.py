"""The benchmark's reference arm on the CPU: one JSON line with the keys the
harness reads (a tiny grid, so it runs in seconds without a GPU)."""
import json
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--grid", "8",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "Gcell-updates/s"
    assert d["warmup"] == 3 and d["steps"] >= 2 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    # both arms describe the workload with the same dict
    import bench
    bench.WORKLOAD["n"] = 8
    assert d["config"] == bench.bench_config(bench.make_problem(nt=5), 1)
