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
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(ROOT / "include")]
SOURCES = ["capi.cu", "conv.cu", "solve.cu", "setup.cpp", "noalloc.cu", "stats.cu"]


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
    drv_src = CSRC / "driver.cpp"
    if drv_src.exists() and (force or _stale(DRIVER, [drv_src, LIB, ROOT / "include" / "chgpu.h"])):
        _run(["g++", "-O2", "-std=c++17", "-pthread", "-I", str(ROOT / "include"), str(drv_src), "-o", str(DRIVER),
              f"-L{OUT}", "-lchgpu", f"-Wl,-rpath,{OUT}"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
