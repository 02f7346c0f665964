"""Build recipe for libseidart_gpu.so (sm_103a only).

Every kernel file is compiled three times: the FP64 drop-in build with
``--fmad=false`` (so each FP64 expression keeps the reference's rounding
sequence), the fast FP64 build (FP64 fields, reciprocals and FMA
contraction) and the FP32 fast build with FMA contraction.  Host code is built
with ``-ffp-contract=off`` so host-side coefficient set-up matches the CPU
restatement bit for bit on x86 and on Arm.  Objects compile in parallel; the
library is linked in-tree next to this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
LIB = PKG / "libseidart_gpu.so"
BUILD = PKG.parent / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", str(INCLUDE)]
# (source, precision) pairs; precision None = compiled once
DUAL = ["seismic2.cu", "electromag2.cu", "seismic25.cu", "electromag25.cu", "seismic3.cu", "electromag3.cu"]
SINGLE = ["solver.cu", "seismic3_fast.cu", "seismic3_tma.cu", "seismic3_cell.cu", "seismic3_bulk.cu", "fileio.cu", "batch.cu", "adjoint.cu", "adjoint_em.cu", "noalloc.cu", "material.cu", "planewave.cu", "matidx.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libseidart_gpu.so")


def _jobs() -> list[tuple[list[str], Path]]:
    nvcc = _nvcc()
    jobs = []
    for src in DUAL:
        for prec in ("f64", "f64x", "f32"):
            obj = BUILD / f"{Path(src).stem}.{prec}.o"
            flags = {"f64": ["--fmad=false", "-DSEIDART_REAL=double"],
                     "f64x": ["-DSEIDART_REAL=double", "-DSEIDART_FAST64"],
                     "f32": ["-DSEIDART_REAL=float", "-DSEIDART_FP32"]}[prec]
            jobs.append(([nvcc, *ARCH, *COMMON, *flags, "-c", str(CSRC / src), "-o", str(obj)], obj))
    for src in SINGLE:
        if not (CSRC / src).exists():
            continue
        obj = BUILD / f"{Path(src).stem}.o"
        jobs.append(([nvcc, *ARCH, *COMMON, "-c", str(CSRC / src), "-o", str(obj)], obj))
    return jobs


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link libseidart_gpu.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    jobs = _jobs()
    todo = []
    for cmd, obj in jobs:
        src = Path(cmd[cmd.index("-c") + 1])
        if force or _stale(obj, [src, *headers]):
            todo.append((cmd, obj))

    def run(job):
        cmd, obj = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {obj.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    if todo:
        with ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(run, todo))
    objs = [str(obj) for _, obj in jobs]
    if force or todo or not LIB.exists() or _stale(LIB, [Path(o) for o in objs]):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(LIB), *objs, "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    exe = PKG / "seidartfdtd"
    main_c = CSRC / "seidartfdtd_main.c"
    if main_c.exists() and (force or not exe.exists() or _stale(exe, [LIB, main_c])):
        cmd = [_nvcc(), *ARCH, "-o", str(exe), str(main_c), "-L", str(PKG), "-lseidart_gpu",
               "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"seidartfdtd link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
