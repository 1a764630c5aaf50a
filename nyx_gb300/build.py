"""Build libnyxpm.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled separately (in parallel) and linked into
nyx_gb300/libnyxpm.so.  The FP64 units are compiled with --fmad=false so that
no multiply-add is contracted: their results then round exactly as the
expressions are written.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnyxpm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no contraction either (aarch64 g++ would fuse multiply-adds by default)
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
          "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
# unit -> extra flags
UNITS = {
    "pm_api.cu": ["--fmad=false"],
    "pm_particles.cu": ["--fmad=false"],
    "pm_multigrid.cu": ["--fmad=false"],
    "pm_mixed.cu": [],
    "pm_ensemble.cu": [],
    "pm_noalloc.cu": ["--fmad=false"],
    "pm_amr.cu": ["--fmad=false"],
    "pm_probe.cu": [],
    "pm_io.cpp": [],
    "pm_vismf.cpp": [],
    "pm_particle_io.cpp": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(unit: str, flags: list[str], verbose_ptxas: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(os.path.dirname(HERE), "include", "nyxpm.h")
    return os.path.getmtime(hdr) > t


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose_ptxas), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
