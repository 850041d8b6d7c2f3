"""Builds libchgpu.so (the CUDA step library) and the C++ driver in-tree.

nvcc compiles each translation unit for sm_103a in parallel, then links a
shared library into channel_gb300/_build/.  No CMake; the recipe is this
file.  Run ``python -m channel_gb300.build`` or call ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libchgpu.so"
DRIVER = OUT / "channel_gb300"
OUT2BIN = OUT / "out2bin"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(ROOT / "include")]
SOURCES = ["capi.cu", "conv.cu", "convf_f32.cu", "convf_f64.cu", "convf_dd.cu", "solve.cu", "setup.cpp", "noalloc.cu", "stats.cu", "export.cu", "mlp.cu", "peaks.cu",
           "closure.cu", "tke.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "chgpu.h"]
    objs = []
    jobs = []
    nv = nvcc()
    for src in SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nv, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
            if ptxas_info and s.suffix == ".cu":
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose or ptxas_info:
                    print(out, file=sys.stderr)
    if force or _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    # host programs over the C ABI: the driver (channel.f90) and the exporter (out2bin.f90)
    host_jobs = []
    for src, exe in (("driver.cpp", DRIVER), ("out2bin.cpp", OUT2BIN)):
        s = CSRC / src
        if force or _stale(exe, [s, LIB, CSRC / "hostio.h", ROOT / "include" / "chgpu.h"]):
            host_jobs.append(["g++", "-O2", "-std=c++17", "-pthread", "-I", str(ROOT / "include"), str(s), "-o",
                              str(exe), f"-L{OUT}", "-lchgpu", f"-Wl,-rpath,{OUT}"])
    if host_jobs:
        with cf.ThreadPoolExecutor(max_workers=len(host_jobs)) as ex:
            list(ex.map(_run, host_jobs))
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
