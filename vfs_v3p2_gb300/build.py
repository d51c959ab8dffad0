"""Builds the CUDA library libvfs_gb300.so for sm_103a (GB300) in-tree.

Each translation unit is compiled in parallel with one -gencode; the setup
and per-step FP64 units (k_setup.cu, k_proj.cu) are compiled with
--fmad=false so that their arithmetic matches the reference's uncontracted
double operations bit for bit.  Output: vfs_v3p2_gb300/_lib/libvfs_gb300.so
(git-ignored, rebuilt on each machine because the GPU host is aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shlex
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libvfs_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "k_setup.cu": ["--fmad=false"],
    "k_proj.cu": ["--fmad=false"],
    "k_mg.cu": [],
    "k_group.cu": [],
    "k_smooth_tma.cu": [],
    "k_krylov.cu": [],
    "vfs_host.cu": [],
}
EXTRA_UNITS: dict = {}


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    # VFS_NVCC_FLAGS: extra nvcc flags (compile-time tuning knobs such as
    # -DVFS_SMOOTH_PF_FACE=2; rebuild with --force after changing it)
    extra = shlex.split(os.environ.get("VFS_NVCC_FLAGS", ""))
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", SRC, "-I", os.path.join(ROOT, "include")] + ARCH + extra


def _compile(unit: str, extra, verbose: bool):
    src = os.path.join(SRC, unit)
    obj = os.path.join(OUT_DIR, unit.replace(".cu", ".o"))
    cmd = [nvcc(), "-c", src, "-o", obj] + _flags() + list(extra)
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(SRC):
        if os.path.getmtime(os.path.join(SRC, f)) > t:
            return True
    hdr = os.path.join(ROOT, "include", "vfs_gpu.h")
    return os.path.getmtime(hdr) > t or os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    units = dict(UNITS)
    units.update(EXTRA_UNITS)
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        futs = {ex.submit(_compile, u, f, verbose): u for u, f in units.items()}
        objs, logs = [], []
        for fu in cf.as_completed(futs):
            o, log = fu.result()
            objs.append(o)
            logs.append((futs[fu], log))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + sorted(objs) + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        for u, log in sorted(logs):
            print(f"== {u}\n{log}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
