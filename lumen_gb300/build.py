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
SOURCES = ["abi.cu", "bvh_build.cu", "traverse.cu", "path.cu", "diag.cu", "film.cu", "adjoint.cu", "vcm.cu", "sppm.cu",
           "restir.cu", "bdpt.cu"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-Xcompiler", "-ffp-contract=off",
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
    build_host(lib)
    return lib


HOST_SOURCES = ["lumen_scene.cpp", "mitsuba_xml.cpp", "integrator.cpp", "host_capi.cpp"]


def build_host(lib: str) -> str:
    """liblgb_host.so (scene loading + Integrator mirror, plain C++ over the C ABI) and the lgb_render CLI."""
    hdir = os.path.join(HERE, "host")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + hdir]
    objs = [os.path.join(OUT, "host_" + s.replace(".cpp", ".o")) for s in HOST_SOURCES]
    jobs = [[NVCC, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", *inc, "-c",
             os.path.join(hdir, s), "-o", o] for s, o in zip(HOST_SOURCES, objs)]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    host = os.path.join(OUT, "liblgb_host.so")
    rpath = ["-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
    _run([NVCC, "-shared", "--cudart", "static", "-o", host, *objs, "-L" + OUT, "-llgb", *rpath])
    _run([NVCC, "-O2", "-std=c++17", *inc, os.path.join(hdir, "lgb_render.cpp"), "-o", os.path.join(OUT, "lgb_render"),
          "-L" + OUT, "-llgb_host", "-llgb", *rpath])
    return host
