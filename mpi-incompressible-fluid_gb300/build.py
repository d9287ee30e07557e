"""Build recipe of the mifgpu shared library (sm_103a).

Compiles every translation unit under csrc/ with nvcc in parallel and links
them into libmifgpu.so next to this file (in-tree, git-ignored). Re-running is
incremental: objects newer than all sources are reused.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "libmifgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps separate multiplies and adds (-ffp-contract=off): the export
# writers reproduce the reference's arithmetic bit for bit on x86 and Arm hosts.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the mifgpu CUDA library cannot be built")


def _newest(paths) -> float:
    return max(os.path.getmtime(p) for p in paths)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile and link libmifgpu.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "mifgpu.h")]
    hdr_time = _newest(headers)
    flags = NVCC_FLAGS + list(extra_flags or [])

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            return obj
        cmd = [nvcc] + flags + ["-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(sources), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, sources))
    stamp = os.path.join(BUILD, "lib.stamp")
    if not os.path.exists(LIB) or not os.path.exists(stamp) or os.path.getmtime(stamp) < _newest(objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        with open(stamp, "w") as f:
            f.write(platform.machine() + "\n")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
