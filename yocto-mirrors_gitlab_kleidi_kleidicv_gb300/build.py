"""Build recipe of the GB300 library: nvcc for the CUDA units (sm_103a only),
g++ for host units, linked into libkleidicv_gpu.so next to this file.

    python build.py [--force] [--jobs N]

Translation units are compiled in parallel and only when a source or header
is newer than its object.  cudart is linked statically so the library loads
(and reports "no device") on machines without a GPU.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkleidicv_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-diag-suppress", "1160", *ARCH]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-ffp-contract=off"]


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(CSRC, "*.inc")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj, src, hdr_mtime):
    return not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_mtime)


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return cmd[-1]


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + CSRC, "-I" + INCLUDE, "-I" + os.path.join(cuda, "include")]
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    cmds, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hdr_mtime):
            cmds.append([nvcc, *NVCC_FLAGS, *inc, "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hdr_mtime):
            cmds.append(["g++", *CXX_FLAGS, *inc, "-pthread", "-c", src, "-o", obj])
    if cmds:
        jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 1))
        # Longest units first so the slowest compile starts immediately.
        cmds.sort(key=lambda c: 0 if "fused_sigma_21" in c[-3] or "fused_sigma_15" in c[-3] else 1)
        with cf.ThreadPoolExecutor(jobs) as ex:
            for done in ex.map(_compile, cmds):
                if verbose:
                    print("built", os.path.basename(done), file=sys.stderr)
    if force or cmds or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        link = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", LIB, *objs, "-cudart", "static",
                "-lpthread"]
        _compile(link)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    a = ap.parse_args()
    print(build(a.force, a.jobs, verbose=True))
