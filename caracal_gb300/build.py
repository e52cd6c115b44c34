"""Compile the CUDA engine (sm_103a) into an in-tree shared library.

One nvcc process per translation unit (run in parallel), one -gencode; the
library is rebuilt only when a source under ``csrc/`` or ``include/`` is
newer than it.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libcaracal_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build caracal_gb300")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> tuple[str, str]:
    obj = os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o")
    # host code without FMA contraction: its set-up arithmetic (the QMDFF
    # reader's coordination numbers and C6) then rounds as the Python host
    # does on both x86_64 and aarch64
    cmd = [nvcc_path(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
           "-ffp-contract=off", "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n" + res.stdout + res.stderr)
    return obj, res.stdout + res.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every csrc/*.cu in parallel (one process each), then link."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as pool:
        results = list(pool.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc_path(), ARCH, "-shared", "-o", tmp] + [o for o, _ in results]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    if verbose:
        for _, log in results:
            print(log)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
