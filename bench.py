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
  cpu_baseline  the CPU restatement (reference production flags, OpenMP) on a
            bounded sample of the same workload

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

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
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


def make_problem(nt=None):
    from seidart_gpu import models
    w = WORKLOAD
    return models.seismic3_layers(n=w["n"], cpml=w["cpml"], nt=nt or w["nt"], seed=w["seed"])


def kernel_bytes(p, box_cells: int) -> dict:
    """Algorithmic bytes per launch (FP32): every array the kernel must touch,
    read or written once; CPML memories and coefficients only on the CPML
    shell (outside the inert interior box)."""
    n = p.ncell
    shell = n - box_cells
    stress = WORD * (42 * n + 78 * shell)   # v 3 + C 21 + gamma 6 + sigma R+W 12; shell: 36 memories R+W + 6 coefficients
    velocity = WORD * (13 * n + 24 * shell)  # sigma 6 + rho 1 + v R+W 6; shell: 9 memories R+W + 6 coefficients
    # z-marching kernels (default) and one-thread-per-cell kernels
    return {"s3c_stress": stress, "s3c_velocity": velocity, "s3f_stress": stress, "s3f_velocity": velocity,
            "s3t_stress": stress, "s3b_stress": stress}


def step_bytes(p, box_cells: int) -> int:
    """Per-step algorithmic bytes of the whole leapfrog step: 9 fields read and
    written once, 21 C_ij + rho + 6 gamma read once (46 words), plus 45
    memories R+W and 6 CPML coefficients on shell cells (96 words)."""
    shell = p.ncell - box_cells
    return WORD * (46 * p.ncell + 96 * shell)


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
    st.step(1)  # warm-up (page-in of the 30 GB working set)
    t1 = time.perf_counter() - t0
    k = int(max(2, min(args.steps, 90.0 / max(t1, 1e-3))))
    t0 = time.perf_counter()
    st.step(k)
    dt = time.perf_counter() - t0
    val = p.ncell * k / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": k, "warmup": 1, "ms_per_step": 1e3 * dt / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded layered orthotropic model)",
            "config": {"workload": f"seismic3 {WORKLOAD['n']}^3+16 CPML ({p.nx}^3 padded), reference CPU loops",
                       "grid": [p.nx, p.ny, p.nz], "seed": WORKLOAD["seed"]},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": orc.load("omp").oracle_threads(), "kind": "port",
                             "sample": f"{k} of {args.steps} requested full time steps of the {p.nx}^3 grid after 1 warm-up step (FP64, OpenMP)"},
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
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
    kb = kernel_bytes(p, box_cells)
    kernels = prof["kernels"]
    dom = max((k for k in kernels if k in kb), key=lambda k: kernels[k]["ms"])
    avg_ms = kernels[dom]["ms"] / kernels[dom]["launches"]
    achieved = kb[dom] / (avg_ms / 1e3) / 1e9
    sb = step_bytes(p, box_cells)
    step_gbs = sb * args.steps / (ms_total / 1e3) / 1e9
    launches = sum(v["launches"] for v in kernels.values())
    fp32_fields = s.get_fields()
    tr32, _ = s.traces()
    s.close()

    extra = {}
    if not args.no_fp64 and rank == 0:
        # FP64 drop-in path on the same workload and the FP32-vs-FP64 error
        s64 = sg.Solver(p, sg.FP64)
        s64.step(args.warmup)
        s64.sync()
        k64 = min(args.steps, 40)
        pr64 = s64.profile(k64)
        s64.step(args.steps - k64)
        s64.sync()
        tr64, _ = s64.traces()
        f64 = s64.get_fields()
        s64.close()
        extra["fp64_plain"] = {"value": p.ncell * k64 / (pr64["total_ms"] / 1e3) / 1e9, "unit": UNIT,
                               "steps": k64}
        extra["fp32_vs_fp64"] = {
            "traces_rel_l2": float(np.linalg.norm(tr32 - tr64) / max(np.linalg.norm(tr64), 1e-300)),
            "vz_rel_l2": float(np.linalg.norm(fp32_fields[2] - f64[2]) / max(np.linalg.norm(f64[2]), 1e-300)),
            "steps": args.warmup + args.steps}
        extra["fp32_speedup_vs_fp64"] = value / world / extra["fp64_plain"]["value"]

    e2e = None
    if not args.no_e2e:
        # through the C ABI with host buffers: one full reference-length run
        pe = dataclasses.replace(p, time_steps=WORKLOAD["nt"], src={k: v[:WORKLOAD["nt"]] for k, v in p.src.items()})
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        out = sg.run(pe, sg.FP32)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        barrier()
        model_bytes = sum(a.nbytes for a in pe.model_list())
        src_bytes = sum(a.nbytes for a in pe.src_list() if a is not None)
        f_bytes = sum(a.nbytes for a in pe.field_list())
        tr_bytes = out["traces"].nbytes + out["norms"].nbytes
        e2e = {"value": world * pe.ncell * pe.time_steps / te / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int((model_bytes + src_bytes + f_bytes) / pe.time_steps),
               "d2h_bytes_per_step": int((f_bytes + tr_bytes) / pe.time_steps),
               "steps": pe.time_steps, "seconds": te,
               "note": "seidart_run on host FP64 buffers: upload+FP32 conversion of the model, 1500 steps, "
                       "copy-back of final fields, traces and norms"}

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        cpu = cpu_baseline_sample(p)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 5-layer rotated-orthotropic model, Ricker force source)",
            "config": {"workload": f"seismic3 anisotropic elastic, {WORKLOAD['n']}^3 interior + 16 CPML ({p.nx}^3 padded), FP32",
                       "grid": [p.nx, p.ny, p.nz], "cells": p.ncell, "receivers": 1024, "seed": WORKLOAD["seed"],
                       "l2": "inputs larger than L2 (about 14 GB moved per step vs 129 MB L2)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": None,
                         "algorithmic_bytes_per_launch": kb[dom], "avg_launch_ms": avg_ms},
            "step_roofline": {"achieved": step_gbs, "frac": step_gbs / hbm, "bytes_per_step": sb},
            "kernels": kernels,
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "wall_s_timed": wall,
            **extra,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
