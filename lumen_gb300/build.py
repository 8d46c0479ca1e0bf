"""In-tree build of liblgb.so: one nvcc job per translation unit (in parallel), then one link.

Flags: sm_103a only, -O3, -lineinfo, no fast-math (IEEE division and square root), and -fmad=false so
that separate multiplies and adds are never fused behind the source's back; the traversal box tests
call fmaf explicitly where fusing is wanted.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
SOURCES = ["abi.cu", "bvh_build.cu", "traverse.cu", "path.cu", "diag.cu"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-I" + os.path.join(ROOT, "include"), "-I" + SRC]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_library(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    objs = [os.path.join(OUT, s.replace(".cu", ".o")) for s in SOURCES]
    jobs = [[NVCC, *ARCH, *CFLAGS, "-c", os.path.join(SRC, s), "-o", o] for s, o in zip(SOURCES, objs)]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr)
    lib = os.path.join(OUT, "liblgb.so")
    _run([NVCC, *ARCH, "-shared", "--cudart", "static", "-o", lib, *objs])
    return lib
