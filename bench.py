#!/usr/bin/env python
"""Benchmark: Gcell-updates/s of the 3D anisotropic elastic CPML-FDTD step.

Workload: the 3D configuration -- 320^3 interior + 16-cell CPML (352^3 padded
cells), five rotated orthotropic layers (21 C_ij), FP32 fields, seeded
synthetic model.  One bench "step" is one leapfrog time step of the whole
grid (stress half-step + velocity half-step, source, Dirichlet faces, norms,
32x32 receiver gather).

  value     Gcell-updates/s over K timed steps, model and state resident in HBM
  e2e       the same metric through the C ABI with host buffers (seidart_run:
            model upload + conversion, a full 1500-step run, copy-back of the
            final fields and traces)
  roofline  dominant kernel: algorithmic bytes per launch / its CUDA-event time
            (the layered model runs the material-indexed stress kernel: one
            byte per cell instead of 27 coefficient words, counted as such;
            per_cell_layout times the per-cell arrays on the same steps)
  cpu_baseline  the CPU restatement (reference production flags, OpenMP) on a
            bounded sample of the same workload
  configs_2d  the two 2D workloads at full length: seismic2 256^2 + 20 CPML
            (2000 steps; FP64 plain, FP32 and the CPU restatement) and
            electromag2 1024^2 + 20 CPML (4000 steps; FP64 and FP32)
  families  seismic25, electromag25 (1024^2) and electromag3 (256^3) in the
            three precisions
  batched   the ragged multi-model 2D workload: 64 seismic2 models with nx, nz
            in [256, 1024], 3000 steps, one persistent launch per graph chunk
            with autotuned tiles; beside it the same models run one by one
  fwi       the 2D elastic misfit gradient: 512^2 + 20 CPML, 3000 steps, 16
            shots, 128 receivers, Gaussian anomaly target; gradient time
            against one forward and a central-difference check of the
            gradient at 8 seeded cells (FP64 forward runs, one shot)

``--impl reference`` times the CPU restatement of the reference time loops
(oracle/, OpenMP, all host cores) on the same workload instead.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "seidart-backend_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-updates/s & % HBM peak, FP32 vs FP64 plain; FWI gradients/s at stated err"
UNIT = "Gcell-updates/s"
WORKLOAD = dict(n=320, cpml=16, nt=1500, seed=2)
WORD = 4  # FP32 bytes per word


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int, interval_ms: int = 20):
        self.gpu = gpu
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def bench_config(p, world: int = 1) -> dict:
    """The workload description both arms print (same keys and values; the
    arithmetic type is the line's own ``dtype``)."""
    return {"workload": f"seismic3 anisotropic elastic, {WORKLOAD['n']}^3 interior + {WORKLOAD['cpml']} CPML "
                        f"({p.nx}^3 padded cells), 5 rotated orthotropic layers",
            "grid": [p.nx, p.ny, p.nz], "cells": p.ncell, "receivers": 1024, "seed": WORKLOAD["seed"],
            "l2": "inputs larger than L2 (about 14 GB moved per step vs 129 MB L2)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def make_problem(nt=None):
    from seidart_gpu import models
    w = WORKLOAD
    return models.seismic3_layers(n=w["n"], cpml=w["cpml"], nt=nt or w["nt"], seed=w["seed"])


# DRAM traffic / algorithmic bytes of one launch: ncu's dram__bytes_read.sum +
# dram__bytes_write.sum of one launch of each kernel on the 224^3 case (a
# full-size launch is too large for a multi-pass capture), divided by that
# launch's algorithmic bytes; the bench scales it to its own launch by the
# algorithmic bytes.
TRAFFIC_RATIO = {"s3x_stress": 1.081, "s3b_stress": 1.113, "s3c_velocity": 1.146, "s3p_velocity": 1.153,
                 "s3x_stress/indexed-merged": 1.088, "s3x_stress/indexed-merged-cpml": 1.066}


def kernel_bytes(p, box_cells: int, indexed: bool = False, mems: int = 36, cpmlidx: bool = False) -> dict:
    """Algorithmic bytes per launch (FP32): every array the kernel must touch,
    read or written once; CPML memories and coefficients only on the CPML
    shell (outside the inert interior box).  `indexed`: the stress kernel
    reads the material-indexed layout -- one byte per cell instead of the
    21 C_ij and 6 attenuation factors (the table of tuples is a few KB).
    `mems`: stress-loop memories it advances (36, or 21 when the loops that
    share a derivative stencil and its coefficients share the memory).
    `cpmlidx`: shell cells read one C-PML byte instead of the six C-PML
    coefficient grids."""
    n = p.ncell
    shell = n - box_cells
    cp_w, cp_b = (0, 1) if cpmlidx else (6, 0)  # C-PML coefficients per shell cell: words, bytes
    sh = 2 * mems + cp_w  # shell: memories R+W + the C-PML coefficients
    stress = WORD * (42 * n + sh * shell) + cp_b * shell   # v 3 + C 21 + gamma 6 + sigma R+W 12
    if indexed:
        stress = WORD * (15 * n + sh * shell) + n + cp_b * shell  # v 3 + sigma R+W 12 + one material byte
    # sigma 6 + rho 1 + v R+W 6; shell: 9 memories R+W + the C-PML coefficients
    velocity = WORD * (13 * n + (18 + cp_w) * shell) + cp_b * shell
    # the fused step does both half-steps: the whole step's algorithmic bytes
    return {"s3c_stress": stress, "s3c_velocity": velocity, "s3x_velocity": velocity, "s3p_velocity": velocity,
            "s3f_stress": stress, "s3f_velocity": velocity,
            "s3t_stress": stress, "s3b_stress": stress, "s3x_stress": stress,
            "s3w_step": step_bytes(p, box_cells)}


def step_bytes(p, box_cells: int, indexed: bool = False, mems: int = 36, cpmlidx: bool = False) -> int:
    """Per-step algorithmic bytes of the whole leapfrog step: 9 fields read and
    written once, 21 C_ij + rho + 6 gamma read once (46 words), plus 45
    memories R+W and 6 CPML coefficients on shell cells (96 words).
    `indexed`: one material byte per cell in place of the 27 coefficient
    words (19 words + 1 byte per cell); `mems` = 21: the stress loops' 36
    memories held as 21 (30 memories R+W + 6 coefficients = 66 words);
    `cpmlidx`: one C-PML byte per shell cell instead of the six coefficient
    words."""
    shell = p.ncell - box_cells
    sh = 2 * (mems + 9) + (0 if cpmlidx else 6)
    extra = shell if cpmlidx else 0
    if indexed:
        return WORD * (19 * p.ncell + sh * shell) + p.ncell + extra
    return WORD * (46 * p.ncell + sh * shell) + extra


def interior_box_cells(p) -> int:
    # mirrors the runtime's box: nominal [cpml, n-cpml) minus the one-cell
    # layer the half-grid CPML profile reaches on each high side
    dims = [p.nx, p.ny, p.nz]
    vol = 1
    for d in dims:
        vol *= max(0, d - 2 * p.cpml - 1)
    return vol


def run_reference(args, rank: int) -> None:
    """CPU restatement of the reference loops, OpenMP on all host cores.  Each
    step is one full time step of the same grid; when K steps would run past
    about 90 s, only the first steps that fit are timed (the value is a rate)."""
    if rank != 0:
        return
    from oracle import oracle as orc
    nthreads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(nthreads))
    p = make_problem(nt=args.warmup + args.steps + 1)
    st = orc.OracleState(p, kind="omp")
    t0 = time.perf_counter()
    st.step(args.warmup)  # warm-up steps (page-in of the 30 GB working set)
    t1 = (time.perf_counter() - t0) / args.warmup
    k = int(max(2, min(args.steps, 90.0 / max(t1, 1e-3))))
    t0 = time.perf_counter()
    st.step(k)
    dt = time.perf_counter() - t0
    val = p.ncell * k / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": k, "warmup": args.warmup, "ms_per_step": 1e3 * dt / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded layered orthotropic model)",
            "config": bench_config(p, args.gpus),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": orc.load("omp").oracle_threads(), "kind": "port",
                             "sample": f"{k} of {args.steps} requested full time steps of the {p.nx}^3 grid after {args.warmup} warm-up steps (FP64, OpenMP)"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(p=None, budget_s: float = 20.0) -> dict:
    """Time the OpenMP CPU restatement on a bounded sample of the workload:
    the same model, as many full time steps as fit ~budget_s."""
    from oracle import oracle as orc
    p = make_problem(nt=64) if p is None else p
    st = orc.OracleState(p, kind="omp")
    t0 = time.perf_counter()
    st.step(1)
    t1 = time.perf_counter() - t0
    n = int(max(1, min(60, budget_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    st.step(n)
    dt = time.perf_counter() - t0
    return {"value": p.ncell * n / dt / 1e9, "unit": UNIT, "cores": orc.load("omp").oracle_threads(), "kind": "port",
            "sample": f"{n} full time steps of the {p.nx}^3 grid after 1 untimed step (FP64, OpenMP, reference flags)"}


def _timed_run(p, precision, warm: int = 10, want_fields: bool = False) -> dict:
    """Whole run of problem p through the Solver API: `warm` untimed steps,
    then the remaining steps timed with CUDA events on the solver's stream."""
    import torch
    import seidart_gpu as sg
    st = torch.cuda.Stream()
    with sg.Solver(p, precision) as s:
        s.set_stream(st.cuda_stream)
        s.step(warm)
        s.sync()
        l0 = s.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        s.step(p.time_steps - warm)
        e1.record(st)
        s.sync()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        tr, _ = s.traces()
        launches = s.launches - l0
        fields = s.get_fields() if want_fields else None
    return {"ms": ms, "steps": p.time_steps - warm, "traces": tr, "launches": launches, "fields": fields}


def bench_2d_configs() -> dict:
    """The two 2D workloads, each run for its full length.

    seismic2 two-layer (256^2 + 20 CPML, 2000 steps): FP64 plain and FP32 on
    the GPU, and the OpenMP CPU restatement (reference flags, all host
    cores) on the same 2000 steps.  electromag2 blocks (1024^2 + 20 CPML,
    12 blocks, 4000 steps): FP64 and FP32.  Both also run the fast FP64 build
    (FP64 fields, reciprocals and FMA contraction).  Bytes per step follow the
    algorithmic count (seismic2: 20 words per cell + 30 per CPML cell;
    electromag2: 12 + 14); both working sets fit in the 129 MB L2 (2.4 MB
    and 59 MB per FP32 step), so the fraction of the HBM peak can pass 1."""
    import seidart_gpu as sg
    from oracle import oracle as orc
    from seidart_gpu import models
    hbm, _ = peaks()

    def rel(a, b):
        return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))

    out = {}
    cases = [("seismic2_256", models.seismic2_two_layer(), 256, 20, 30),
             ("electromag2_1024", models.electromag2_blocks(nblocks=12), 1024, 12, 14)]
    for name, p, n_int, w_cell, w_shell in cases:
        shell = p.ncell - n_int * n_int
        r = {"grid": [p.nx, p.nz], "cells": p.ncell, "steps": p.time_steps, "seed": p.meta.get("seed")}
        runs = {}
        for prec, word, key in ((sg.FP64, 8, "fp64_plain"), (sg.FP64_FAST, 8, "fp64_fast"), (sg.FP32, 4, "fp32")):
            t = _timed_run(p, prec)
            runs[key] = t
            gbs = word * (w_cell * p.ncell + w_shell * shell) * t["steps"] / (t["ms"] / 1e3) / 1e9
            r[key] = {"value": p.ncell * t["steps"] / (t["ms"] / 1e3) / 1e9, "unit": UNIT,
                      "ms_per_step": t["ms"] / t["steps"], "algorithmic_gbs": gbs, "frac_of_measured_hbm": gbs / hbm,
                      "gpu_launches": t["launches"]}
        r["fp32_vs_fp64_traces_rel_l2"] = rel(runs["fp32"]["traces"], runs["fp64_plain"]["traces"])
        r["fp64_fast_vs_fp64_traces_rel_l2"] = rel(runs["fp64_fast"]["traces"], runs["fp64_plain"]["traces"])
        r["fp32_speedup_vs_fp64"] = r["fp32"]["value"] / r["fp64_plain"]["value"]
        if name.startswith("seismic2"):
            st = orc.OracleState(p, kind="omp")
            t0 = time.perf_counter()
            st.step(p.time_steps)
            dt = time.perf_counter() - t0
            r["cpu_restatement"] = {"value": p.ncell * p.time_steps / dt / 1e9, "unit": UNIT,
                                    "cores": orc.load("omp").oracle_threads(), "kind": "port", "seconds": dt,
                                    "sample": f"all {p.time_steps} steps (FP64, OpenMP, reference flags)"}
            r["fp64_vs_cpu_traces_rel_l2"] = rel(runs["fp64_plain"]["traces"], st.result()["traces"])
            r["fp64_speedup_vs_cpu"] = r["fp64_plain"]["value"] / r["cpu_restatement"]["value"]
        out[name] = r
    return out


def bench_families() -> dict:
    """The solvers the headline and 2D legs do not time: seismic25 and
    electromag25 (2.5D, complex fields) on 1024^2 + 20 CPML for 400 steps
    and electromag3 on 256^3 + 10 CPML for 200 steps, each in FP64 exact,
    fast FP64 and FP32, with the FP32 and fast-FP64 errors against exact FP64
    on the final fields (on these grids and step counts the wave has not yet
    reached the receiver lines, whose FP64 samples are leading-edge values
    far below FP32's range)."""
    import seidart_gpu as sg
    from seidart_gpu import models

    def rel(a, b):
        return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))

    cases = [("seismic25_1024", models.seismic25_two_layer(n=1024, cpml=20, nt=400)),
             ("electromag25_1024", models.electromag25_blocks(n=1024, cpml=20, nt=400)),
             ("electromag3_256", models.electromag3_blocks(n=256, cpml=10, nt=200))]
    out = {}
    for name, p in cases:
        r = {"grid": list(p.shape), "cells": p.ncell, "steps": p.time_steps}
        runs = {}
        for prec, key in ((sg.FP64, "fp64_plain"), (sg.FP64_FAST, "fp64_fast"), (sg.FP32, "fp32")):
            t = _timed_run(p, prec, want_fields=True)
            runs[key] = t
            r[key] = {"value": p.ncell * t["steps"] / (t["ms"] / 1e3) / 1e9, "unit": UNIT,
                      "ms_per_step": t["ms"] / t["steps"], "gpu_launches": t["launches"]}
        ref = np.concatenate([np.asarray(f).ravel() for f in runs["fp64_plain"]["fields"]])
        for key in ("fp32", "fp64_fast"):
            got = np.concatenate([np.asarray(f).ravel() for f in runs[key]["fields"]])
            r[f"{key}_vs_fp64_fields_rel_l2"] = rel(got, ref)
        r["fp64_max_abs_trace"] = float(np.max(np.abs(runs["fp64_plain"]["traces"])))
        out[name] = r
    return out


def bench_plane_wave_3d(nt: int = 200) -> dict:
    """The 3D workload (352^3 cells) with a plane-wave source in place of the
    point force: FP32 on the fast kernels (tiles that meet an injection face
    take the per-cell path, the faces are injected after each velocity
    update) and fast FP64, with the FP32 error on the final fields."""
    import seidart_gpu as sg
    p = make_problem(nt=nt)
    p = dataclasses.replace(p, src={}, plane_wave={"kind": "pw", "wavelet": "gaus1", "frequency": 40.0,
                                                   "x_z_rotation": 20.0, "x_y_rotation": 30.0})
    r = {"grid": list(p.shape), "cells": p.ncell, "steps": p.time_steps,
         "source": "plane wave (gaus1, 40 Hz, rotations x-z 20, x-y 30 degrees)"}
    runs = {}
    for prec, key in ((sg.FP32, "fp32"), (sg.FP64_FAST, "fp64_fast")):
        t = _timed_run(p, prec, want_fields=True)
        runs[key] = t
        r[key] = {"value": p.ncell * t["steps"] / (t["ms"] / 1e3) / 1e9, "unit": UNIT,
                  "ms_per_step": t["ms"] / t["steps"], "gpu_launches": t["launches"]}
    got = np.concatenate([np.asarray(f).ravel() for f in runs["fp32"]["fields"]])
    ref = np.concatenate([np.asarray(f).ravel() for f in runs["fp64_fast"]["fields"]])
    r["fp32_vs_fp64_fast_fields_rel_l2"] = float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))
    return r


def bench_batch(nmodels: int = 64, nt: int = 3000, warm: int = 20) -> dict:
    """Ragged batch: all models advance together; rate over the timed steps."""
    import torch
    import seidart_gpu as sg
    from seidart_gpu import models
    from seidart_gpu.batch import Batch
    ps = models.batch_layered_vti(nmodels=nmodels, nt=nt)
    cells = sum(p.ncell for p in ps)
    t0 = time.perf_counter()
    b = Batch(ps, autotune=True)
    setup = time.perf_counter() - t0
    b.step(warm)
    b.sync()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.step(nt - warm, chunk=500)
    b.sync()
    dt = time.perf_counter() - t0
    cfg = b.config()
    launches = b.launches
    graph_launches = b.graph_launches
    mats = [b.material_count(m) for m in range(len(ps))]
    b.close()
    # the same timed steps with the per-cell coefficient arrays
    os.environ["SEIDART_BATCH_MATIDX"] = "0"
    try:
        bp = Batch(ps, autotune=True)
        bp.step(warm)
        bp.sync()
        t0 = time.perf_counter()
        bp.step(nt - warm, chunk=500)
        bp.sync()
        dtp = time.perf_counter() - t0
        cfgp = bp.config()
        bp.close()
    finally:
        del os.environ["SEIDART_BATCH_MATIDX"]
    # the same models one by one (single-model FP32 solver), a bounded sample
    seq_cells, seq_t = 0, 0.0
    for p in ps[:8]:
        q = dataclasses.replace(p, time_steps=300, src={k: v[:300] for k, v in p.src.items()})
        with sg.Solver(q, sg.FP32) as s1:
            s1.step(20)
            s1.sync()
            t1 = time.perf_counter()
            s1.step(280)
            s1.sync()
            seq_t += time.perf_counter() - t1
            seq_cells += q.ncell * 280
    # algorithmic bytes per step: 20 words per cell + 30 per CPML cell (FP32)
    # with per-cell coefficient arrays; an indexed model reads one material
    # byte per cell instead of its nine stress coefficient words
    hbm, _ = peaks()

    def shell(p):
        return p.ncell - (p.nx - 2 * p.cpml) * (p.nz - 2 * p.cpml)

    step_cell = sum(4 * (20 * p.ncell + 30 * shell(p)) for p in ps)
    step_b = sum((4 * (11 * p.ncell + 30 * shell(p)) + p.ncell) if m > 0 else 4 * (20 * p.ncell + 30 * shell(p))
                 for p, m in zip(ps, mats))
    gbs = step_b * (nt - warm) / dt / 1e9
    gbs_cell = step_cell * (nt - warm) / dtp / 1e9
    return {"value": cells * (nt - warm) / dt / 1e9, "unit": UNIT, "models": nmodels, "cells": cells,
            "algorithmic_gbs": gbs, "frac_of_measured_hbm": gbs / hbm, "bytes_per_step": step_b,
            "materials_per_model": {"min": min(mats), "max": max(mats)},
            "per_cell_layout": {"value": cells * (nt - warm) / dtp / 1e9, "unit": UNIT, "seconds": dtp,
                                "frac_of_measured_hbm": gbs_cell / hbm, "bytes_per_step": step_cell,
                                "tuned": cfgp},
            "steps_timed": nt - warm, "seconds": dt, "setup_s": setup, "tuned": cfg, "gpu_launches": launches,
            "graph_replays": graph_launches,
            "one_by_one": {"value": seq_cells / seq_t / 1e9, "unit": UNIT,
                           "sample": "first 8 models, 280 timed steps each, single-model FP32 solver"},
            "dtype": "f32"}


def bench_fwi(n: int = 512, nt: int = 3000, nshots: int = 16, ncheck: int = 8) -> dict:
    """Misfit gradient over all shots: time against one forward, and central
    differences (relative perturbation 1e-4, FP64 forward runs of shot 0) at
    seeded cells where the shot-0 gradient is large."""
    import seidart_gpu as sg
    from seidart_gpu import models
    from seidart_gpu.fwi import Fwi, Shot, with_model
    an = dict(x=n // 2, z=int(300 * n / 512), sigma=20.0 * n / 512, frac=0.05)
    ref = models.seismic2_two_layer(n=n, cpml=20, nt=nt, nrec=128, rec_z=20, anomaly=an)
    start = models.seismic2_two_layer(n=n, cpml=20, nt=nt, nrec=128, rec_z=20, dt=ref.dt)
    true = with_model(start, **{k: ref.model[k] for k in ("c11", "c33", "c55")})
    xs = np.linspace(1, n, nshots + 2)[1:-1].astype(int)
    shots = [Shot(int(x), 20, start.src["z"]) for x in xs]
    with Fwi(true, shots) as f:
        obs = list(f.model_traces())
    with Fwi(start, shots, obs) as f:
        f.loss()
        t0 = time.perf_counter()
        f.loss()
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        loss, _ = f.gradient()
        t_grad = time.perf_counter() - t0
        launches = f.launches
        every, count = f.checkpointing
    p0 = dataclasses.replace(start, xind=shots[0].xind, zind=shots[0].zind, src={"z": shots[0].srcz})
    t0_ = dataclasses.replace(true, xind=shots[0].xind, zind=shots[0].zind, src={"z": shots[0].srcz})
    s64, o64 = sg.run(p0, sg.FP64)["traces"], sg.run(t0_, sg.FP64)["traces"]
    s32 = sg.run(p0, sg.FP32)["traces"]
    levels = {"residual_rel": float(np.linalg.norm(s64 - o64) / np.linalg.norm(s64)),
              "fp32_rounding_rel": float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64)),
              "note": "shot 0 of this configuration: FP64 start-vs-true trace difference against the FP32 "
                      "forward's own rounding; the anomaly's reflection arrives after the last step, so the "
                      "misfit is below FP32 rounding and the FD check below uses a start model 2% off in "
                      "c11, c33, c55 on the same grid, shots, receivers and steps"}
    # gradient check on shot 0 against FP64 central differences, start model 2% off
    start_fd = with_model(start, **{k: 0.98 * start.model[k] for k in ("c11", "c33", "c55")})
    p0 = dataclasses.replace(start_fd, xind=shots[0].xind, zind=shots[0].zind, src={"z": shots[0].srcz})
    with Fwi(start_fd, shots[:1], obs[:1]) as f:
        _, g = f.gradient()

    def loss64(p):
        tr = sg.run(p, sg.FP64)["traces"]
        return 0.5 * float(np.sum((tr - obs[0]) ** 2))

    rng = np.random.default_rng(7)
    errs = []
    keys = ["c11", "c33", "c55", "rho"]
    for q in range(ncheck):
        key = keys[q % len(keys)]
        a = np.abs(g[key])
        strong = np.argwhere(a >= 0.2 * a.max())
        cell = tuple(strong[rng.integers(len(strong))])
        base = start_fd.model[key]
        h = 1e-4 * base[cell]
        plus, minus = base.copy(order="F"), base.copy(order="F")
        plus[cell] += h
        minus[cell] -= h
        fd = (loss64(with_model(p0, **{key: plus})) - loss64(with_model(p0, **{key: minus}))) / (2 * h)
        errs.append({"param": key, "cell": [int(c) for c in cell], "adjoint": float(g[key][cell]), "fd": fd,
                     "rel_err": abs(float(g[key][cell]) - fd) / abs(fd)})
    # the configuration's own start model (no anomaly): its gradient against
    # central differences of fast-FP64 forward runs (shot 0, 4 cells).  The
    # start-vs-true residual lies below the FP32 rounding of the traces
    # (misfit_levels), so this error states what the FP32 gradient is worth
    # on the configuration as written.
    p0c = dataclasses.replace(start, xind=shots[0].xind, zind=shots[0].zind, src={"z": shots[0].srcz})
    obs64 = sg.run(t0_, sg.FP64_FAST)["traces"]
    with Fwi(start, shots[:1], [obs64]) as f:
        _, gc = f.gradient()

    def loss64c(p):
        tr = sg.run(p, sg.FP64_FAST)["traces"]
        return 0.5 * float(np.sum((tr - obs64) ** 2))

    errs_c = []
    for q, key in enumerate(("c11", "c33", "c55", "rho")):
        a = np.abs(gc[key])
        strong = np.argwhere(a >= 0.2 * a.max())
        cell = tuple(strong[rng.integers(len(strong))])
        base = start.model[key]
        h = 1e-4 * base[cell]
        plus, minus = base.copy(order="F"), base.copy(order="F")
        plus[cell] += h
        minus[cell] -= h
        fd = (loss64c(with_model(p0c, **{key: plus})) - loss64c(with_model(p0c, **{key: minus}))) / (2 * h)
        errs_c.append({"param": key, "cell": [int(c) for c in cell], "adjoint": float(gc[key][cell]), "fd": fd,
                       "rel_err": abs(float(gc[key][cell]) - fd) / max(abs(fd), 1e-300)})
    return {"gradients_per_s": 1.0 / t_grad, "gradient_s": t_grad, "forward_s": t_fwd,
            "cost_vs_forward": t_grad / t_fwd, "loss": loss, "shots": nshots, "grid": [start.nx, start.nz],
            "steps": nt, "checkpoint_every": every, "checkpoints": count, "gpu_launches": launches,
            "misfit_levels": levels,
            "fd_check_config_start_model": {
                "max_rel_err": max(e["rel_err"] for e in errs_c), "cells": errs_c,
                "perturbation": "relative 1e-4, central, fast-FP64 forward (shot 0), observed data from the "
                                "fast-FP64 true model",
                "note": "the configuration's start model: its residual is below FP32 trace rounding, so the FP32 "
                        "adjoint gradient is not resolved there"},
            "fd_check": {"max_rel_err": max(e["rel_err"] for e in errs), "cells": errs,
                         "perturbation": "relative 1e-4, central, FP64 forward (shot 0)",
                         "start_model": "no anomaly, c11 c33 c55 x 0.98"},
            "dtype": "f32 fields, f64 gradient accumulation"}


def bench_fwi_em(n: int = 512, nt: int = 3000, nshots: int = 8, ncheck: int = 6) -> dict:
    """electromag2 misfit gradient (eps, sigma) on the GPR grid of the 2D EM
    configuration's spacing: 512^2 + 20 CPML, 3000 steps, shots along z = 20
    driving Ez, 128 receivers at z = 25; observed data from the background
    plus a Gaussian anomaly (sigma 20 cells, +10% eps11 and eps33, x3
    conductivity) at (256, 150).  Time against one forward, and central
    differences (relative perturbation 1e-4, FP64 forward runs of shot 0) at
    seeded cells where the shot-0 gradient is large."""
    import seidart_gpu as sg
    from seidart_gpu import models
    from seidart_gpu.fwi import Fwi, Shot, with_model
    p = models.electromag2_blocks(n=n, cpml=20, nt=nt, src=(n // 2, 20), nrec=128, rec_z=25, nblocks=0)
    shape = p.shape
    start = with_model(p, e13=np.full(shape, 0.2), s11=np.full(shape, 1e-3), s13=np.full(shape, 1e-4),
                       s33=np.full(shape, 1.5e-3))
    x = np.arange(shape[0])[:, None]
    z = np.arange(shape[1])[None, :]
    g = np.exp(-((x - (n // 2 + 20)) ** 2 + (z - (150 * n // 512 + 20)) ** 2) / (2 * (20.0 * n / 512) ** 2))
    true = with_model(start, e11=start.model["e11"] * (1 + 0.1 * g), e33=start.model["e33"] * (1 + 0.1 * g),
                      s11=start.model["s11"] * (1 + 2 * g), s33=start.model["s33"] * (1 + 2 * g))
    xs = np.linspace(1, n, nshots + 2)[1:-1].astype(int)
    shots = [Shot(int(xx), 20, start.src["z"]) for xx in xs]
    with Fwi(true, shots) as f:
        obs = list(f.model_traces())
    with Fwi(start, shots, obs) as f:
        f.loss()
        t0 = time.perf_counter()
        f.loss()
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        loss, _ = f.gradient()
        t_grad = time.perf_counter() - t0
        launches = f.launches
    # misfit against FP32 rounding on shot 0 (as for the elastic leg), then
    # the central-difference check on a start model whose residual is far
    # above that rounding: eps11, eps33 5% low, sigma11, sigma33 x 1.5
    p0 = dataclasses.replace(start, xind=shots[0].xind, zind=shots[0].zind, src={"z": shots[0].srcz})
    t0_ = dataclasses.replace(true, xind=shots[0].xind, zind=shots[0].zind, src={"z": shots[0].srcz})
    s64, o64 = sg.run(p0, sg.FP64)["traces"], sg.run(t0_, sg.FP64)["traces"]
    s32 = sg.run(p0, sg.FP32)["traces"]
    levels = {"residual_rel": float(np.linalg.norm(s64 - o64) / np.linalg.norm(s64)),
              "fp32_rounding_rel": float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64))}
    start_fd = with_model(start, e11=0.95 * start.model["e11"], e33=0.95 * start.model["e33"],
                          s11=1.5 * start.model["s11"], s33=1.5 * start.model["s33"])
    with Fwi(start_fd, shots[:1], obs[:1]) as f:
        _, gr = f.gradient()
    p0 = dataclasses.replace(start_fd, xind=shots[0].xind, zind=shots[0].zind, src={"z": shots[0].srcz})
    start = start_fd

    def loss64(q):
        tr = sg.run(q, sg.FP64)["traces"]
        return 0.5 * float(np.sum((tr - obs[0]) ** 2))

    rng = np.random.default_rng(8)
    errs = []
    keys = ["e11", "e33", "s11", "s33", "e13", "s13"]
    for q in range(ncheck):
        key = keys[q % len(keys)]
        a = np.abs(gr[key])
        strong = np.argwhere(a >= 0.2 * a.max())
        cell = tuple(strong[rng.integers(len(strong))])
        base = start.model[key]
        h = 1e-4 * abs(base[cell])
        plus, minus = base.copy(order="F"), base.copy(order="F")
        plus[cell] += h
        minus[cell] -= h
        fd = (loss64(with_model(p0, **{key: plus})) - loss64(with_model(p0, **{key: minus}))) / (2 * h)
        errs.append({"param": key, "cell": [int(c) for c in cell], "adjoint": float(gr[key][cell]), "fd": fd,
                     "rel_err": abs(float(gr[key][cell]) - fd) / abs(fd)})
    return {"gradients_per_s": 1.0 / t_grad, "gradient_s": t_grad, "forward_s": t_fwd,
            "cost_vs_forward": t_grad / t_fwd, "loss": loss, "shots": nshots, "grid": [start.nx, start.nz],
            "steps": nt, "gpu_launches": launches, "misfit_levels": levels,
            "fd_check": {"max_rel_err": max(e["rel_err"] for e in errs), "cells": errs,
                         "perturbation": "relative 1e-4, central, FP64 forward (shot 0)",
                         "start_model": "no anomaly, eps11 eps33 x 0.95, sigma11 sigma33 x 1.5"},
            "dtype": "f32 fields, f64 gradient accumulation"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-fwi", action="store_true")
    ap.add_argument("--no-2d", action="store_true", help="skip the seismic2 256^2 and electromag2 1024^2 runs")
    ap.add_argument("--fwi-profile-case", action="store_true",
                    help="run one small misfit gradient (552^2 grid, 4 shots, 240 steps) and exit: the case "
                         "the FWI launch list in profiles/ is captured on")
    ap.add_argument("--batch-profile-case", action="store_true",
                    help="run a small ragged batch (16 models of the batch workload's distribution, 40 steps in "
                         "launches of 20, the autotuned kernel) and exit: the case the batch profile in profiles/ "
                         "is captured on")
    ap.add_argument("--s3-profile-precision", default="fp32", choices=["fp32", "fp64", "fp64fast"],
                    help="precision of --s3-profile-case")
    ap.add_argument("--s3-profile-case", action="store_true",
                    help="run 4 FP32 steps of the 3D workload at --grid (e.g. 192: 224^3 padded cells) through "
                         "the default kernels and exit: the case the 3D kernel profiles in profiles/ are captured on")
    ap.add_argument("--batch-variant", default=None,
                    help="with --batch-profile-case: 'V,B' runs kernel variant V with B CTAs per SM instead of "
                         "the autotuned choice (so a profiler can capture its first launch)")
    ap.add_argument("--grid", type=int, default=WORKLOAD["n"],
                    help="interior cells per axis (default 320: the 3D configuration)")
    args = ap.parse_args()
    WORKLOAD["n"] = args.grid
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.batch_profile_case:
        from seidart_gpu import models
        from seidart_gpu.batch import Batch
        ps = models.batch_layered_vti(nmodels=16, nt=40)
        with Batch(ps, autotune=args.batch_variant is None) as b:
            if args.batch_variant is not None:
                v, bps = (int(x) for x in args.batch_variant.split(","))
                b.set_config(v, bps)
            b.step(40, chunk=20)
            b.sync()
            print(json.dumps({"batch_profile_case": "ok", "config": b.config()}))
        return
    if args.s3_profile_case:
        import seidart_gpu as sg
        p = make_problem(nt=4)
        prec = {"fp32": sg.FP32, "fp64": sg.FP64, "fp64fast": sg.FP64_FAST}[args.s3_profile_precision]
        with sg.Solver(p, prec) as s:
            s.step(4)
            s.sync()
            tr, _ = s.traces()
        print(json.dumps({"s3_profile_case": "ok", "grid": [p.nx, p.ny, p.nz], "trace_max": float(np.abs(tr).max())}))
        return
    if args.fwi_profile_case:
        from seidart_gpu import models
        from seidart_gpu.fwi import Fwi, Shot
        p = models.seismic2_two_layer(n=512, cpml=20, nt=240, nrec=128, rec_z=20)
        shots = [Shot(int(x), 20, p.src["z"]) for x in np.linspace(1, 512, 6)[1:-1].astype(int)]
        with Fwi(p, shots, [np.zeros((240, 2, 128))] * 4) as f:
            loss, _ = f.gradient()
        print(json.dumps({"fwi_profile_case": "ok", "loss": loss}))
        return

    import torch
    import torch.distributed as dist
    import seidart_gpu as sg

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    nt = args.warmup + args.steps
    p = make_problem(nt=max(nt, WORKLOAD["nt"]))
    box_cells = interior_box_cells(p)
    stream = torch.cuda.Stream()
    s = sg.Solver(p, sg.FP32)
    nmat = s.material_count()  # > 0: the stress kernel reads the material-indexed layout
    mems = s.stress_memory_arrays()  # 21: merged stress-loop memories
    ncpml = s.cpml_tuples()  # > 0: indexed C-PML coefficients
    s.set_stream(stream.cuda_stream)
    s.step(args.warmup)
    s.sync()
    clocks = Clocks(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prof = s.profile(args.steps)           # kernels launched with CUDA events between them
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier()
    clk = clocks.stop()
    s.sync()
    ms_total = prof["total_ms"]
    if world > 1:
        t = torch.tensor([ms_total], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    value = world * p.ncell * args.steps / (ms_total / 1e3) / 1e9
    hbm, peak_kind = peaks()
    kb = kernel_bytes(p, box_cells, indexed=nmat > 0, mems=mems, cpmlidx=ncpml > 0)
    kernels = prof["kernels"]
    dom = max((k for k in kernels if k in kb), key=lambda k: kernels[k]["ms"])
    avg_ms = kernels[dom]["ms"] / kernels[dom]["launches"]
    achieved = kb[dom] / (avg_ms / 1e3) / 1e9
    # the capture behind each ratio was of the layout the default solver ran
    # then; a layout without one reports no traffic figure
    traffic_key = (dom if (nmat == 0 and mems == 36 and ncpml == 0) or dom != "s3x_stress"
                   else dom + "/indexed-merged" + ("-cpml" if ncpml > 0 else ""))
    sb = step_bytes(p, box_cells, indexed=nmat > 0, mems=mems, cpmlidx=ncpml > 0)
    step_gbs = sb * args.steps / (ms_total / 1e3) / 1e9
    launches = sum(v["launches"] for v in kernels.values())
    s.close()

    def rel(a, b):
        a, b = np.asarray(a), np.asarray(b)
        return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))

    # the full-length problem: the configuration's 1500 steps from the zero state
    pe = dataclasses.replace(p, time_steps=WORKLOAD["nt"], src={k: v[:WORKLOAD["nt"]] for k, v in p.src.items()})
    e2e, clk_e2e, full32 = None, None, None
    if not args.no_e2e:
        # through the C ABI with host buffers: one full reference-length run
        torch.cuda.synchronize()
        barrier()
        ce = Clocks(local, interval_ms=100)
        ce.start()
        t0 = time.perf_counter()
        with sg.Solver(pe, sg.FP32) as se:   # host FP64 model, sources and initial fields in
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            se.step(pe.time_steps)
            se.sync()
            t2 = time.perf_counter()
            tr_out, nrm_out = se.traces()       # receiver traces and norms out
            f_out = se.get_fields()             # final fields out
            t3 = time.perf_counter()
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        clk_e2e = ce.stop()
        full32 = {"traces": tr_out, "fields": f_out}
        phases = {"setup_s": t1 - t0, "steps_s": t2 - t1, "readback_s": t3 - t2, "teardown_s": t0 + te - t3}
        barrier()
        model_bytes = sum(a.nbytes for a in pe.model_list())
        src_bytes = sum(a.nbytes for a in pe.src_list() if a is not None)
        f0_bytes = sum(a.nbytes for a in pe.given_fields() if a is not None)  # zero initial state: none
        f_bytes = sum(a.nbytes for a in f_out)
        tr_bytes = tr_out.nbytes + nrm_out.nbytes
        e2e = {"value": world * pe.ncell * pe.time_steps / te / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int((model_bytes + src_bytes + f0_bytes) / pe.time_steps),
               "d2h_bytes_per_step": int((f_bytes + tr_bytes) / pe.time_steps),
               "steps": pe.time_steps, "seconds": te, "phases": phases, "clocks": clk_e2e,
               "note": "Solver API on host FP64 buffers: upload and FP32 conversion of the model and sources "
                       "(zero initial state), 1500 steps, copy-back of final fields, traces and norms"}

    extra = {}
    if not args.no_fp64 and rank == 0:
        if full32 is None:
            g = _timed_run(pe, sg.FP32, want_fields=True)
            full32 = {"traces": g["traces"], "fields": g["fields"]}
        # FP64 fields with the fast arithmetic (reciprocals, FMA; within 1e-12
        # of the exact FP64 build): all 1500 steps of the configuration, the
        # FP64 reference the FP32 result is held to
        fx = _timed_run(pe, sg.FP64_FAST, want_fields=True)
        # the exact FP64 drop-in path: its rate over a sample of steps, and its
        # traces against the fast FP64 run's over the same steps
        s64 = sg.Solver(pe, sg.FP64)
        s64.step(args.warmup)
        s64.sync()
        k64 = min(args.steps, 40)
        pr64 = s64.profile(k64)
        s64.sync()
        tr64, _ = s64.traces()
        s64.close()
        n64 = args.warmup + k64
        extra["fp64_plain"] = {"value": p.ncell * k64 / (pr64["total_ms"] / 1e3) / 1e9, "unit": UNIT,
                               "steps": k64, "ms_per_step": pr64["total_ms"] / k64, "dtype": "f64",
                               "build": "exact (IEEE divisions, no FMA contraction; bit-exact with the CPU "
                                        "restatement)"}
        extra["fp64_fast"] = {"value": pe.ncell * fx["steps"] / (fx["ms"] / 1e3) / 1e9, "unit": UNIT,
                              "steps": fx["steps"], "ms_per_step": fx["ms"] / fx["steps"], "dtype": "f64",
                              "traces_rel_l2_vs_fp64": rel(fx["traces"][:n64], tr64),
                              "steps_vs_fp64": n64}
        per_field = [rel(a, b) for a, b in zip(full32["fields"], fx["fields"])]
        extra["fp32_vs_fp64"] = {
            "steps": pe.time_steps, "reference": "fast FP64 build, all steps of the configuration",
            "traces_rel_l2": rel(full32["traces"], fx["traces"]),
            "fields_rel_l2_max": max(per_field),
            "fields_rel_l2": dict(zip(["vx", "vy", "vz", "sxx", "sxy", "sxz", "syy", "syz", "szz"], per_field)),
            "bound": 1e-4}
        extra["fp32_speedup_vs_fp64"] = value / world / extra["fp64_plain"]["value"]
        extra["fp32_speedup_vs_fp64_fast"] = value / world / extra["fp64_fast"]["value"]

    if (nmat > 0 or mems == 21 or ncpml > 0) and rank == 0:
        # the same steps on the reference's data layout -- per-cell
        # coefficient arrays (27 words per cell instead of one material
        # byte) and all 36 stress-loop memories -- on that layout's count
        keep = {k: os.environ.get(k) for k in ("SEIDART_S3_MATIDX", "SEIDART_S3_MERGE", "SEIDART_S3_CPMLIDX")}
        for k in keep:
            os.environ[k] = "0"
        try:
            sp = sg.Solver(p, sg.FP32)
            sp.step(args.warmup)
            sp.sync()
            prp = sp.profile(args.steps)
            sp.sync()
            sp.close()
        finally:
            for k, v in keep.items():
                if v is None:
                    del os.environ[k]
                else:
                    os.environ[k] = v
        msp = prp["total_ms"] / args.steps
        sbp = step_bytes(p, box_cells)
        extra["per_cell_layout"] = {
            "value": p.ncell / (msp / 1e3) / 1e9, "unit": UNIT, "ms_per_step": msp,
            "step_roofline": {"frac": sbp / (msp / 1e3) / 1e9 / hbm, "bytes_per_step": sbp},
            "kernels_ms": {k: v["ms"] / v["launches"] for k, v in prp["kernels"].items()},
            "note": "the staged stress kernel reading the 21 C_ij and 6 attenuation arrays per cell and "
                    "advancing all 36 stress-loop memories"}

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        cpu = cpu_baseline_sample(p)
    legs = {}
    if not args.no_2d and rank == 0:
        legs["configs_2d"] = bench_2d_configs()
        legs["families"] = bench_families()
        legs["plane_wave_3d"] = bench_plane_wave_3d()
    if not args.no_batch and rank == 0:
        legs["batched"] = bench_batch()
    if not args.no_fwi and rank == 0:
        legs["fwi"] = bench_fwi()
        legs["fwi_em"] = bench_fwi_em()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 5-layer rotated-orthotropic model, Ricker force source)",
            "config": bench_config(p, world),
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind,
                         "traffic": TRAFFIC_RATIO[traffic_key] * kb[dom] if traffic_key in TRAFFIC_RATIO else None,
                         "traffic_source": "ncu dram__bytes_read+write of the 224^3 case, scaled by algorithmic bytes",
                         "algorithmic_bytes_per_launch": kb[dom], "avg_launch_ms": avg_ms,
                         "bytes_basis": (f"the layout the kernel reads: {'material-indexed (15 words + 1 byte' if nmat > 0 else 'per-cell coefficient arrays (42 words'} per cell), "
                                         f"{mems} stress-loop memories and {'one C-PML byte' if ncpml > 0 else 'six C-PML words'} per shell cell; the "
                                         "reference's layout (42 + 78 words) is "
                                         f"{kernel_bytes(p, box_cells)[dom] / 1e9:.2f} GB per launch")
                         if dom == "s3x_stress" else "per-cell arrays"},
            "step_roofline": {"achieved": step_gbs, "frac": step_gbs / hbm, "bytes_per_step": sb,
                              "bytes_basis": (f"{'material-indexed: 19 words + 1 byte' if nmat > 0 else 'per-cell arrays: 46 words'} per cell, "
                                              f"{2 * (mems + 9) + (0 if ncpml > 0 else 6)} words{' + 1 byte' if ncpml > 0 else ''} per shell cell; the reference's layout "
                                              f"(46 + 96 words): {step_bytes(p, box_cells) / 1e9:.2f} GB per step")},
            "model_layout": {"materials": nmat, "stress_memory_arrays": mems, "cpml_tuples": ncpml,
                             "stress_coefficients": ("material-indexed: one byte per cell and a table of "
                                                     f"{nmat} FP32 (C_ij, gamma) tuples")
                             if nmat > 0 else "per-cell arrays (21 C_ij + 6 attenuation factors)"},
            **extra,
            "kernels": kernels,
            "wall_s_timed": wall,
            **legs,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
