"""Builds libcoordgpu.so (sm_103a) in-tree with nvcc, no cmake.

    python -m plumed2_gb300.build          # or plumed2_gb300.build.build()

Translation units compile in parallel; k_fp64.cu is compiled with
-fmad=false (the exact FP64 path must not contract multiply-adds) and the
host C++ with -ffp-contract=off (set-up constants must match the reference's
bits).  Output: plumed2_gb300/_build/libcoordgpu.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcoordgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = {
    "k_fp64.cu": ["-fmad=false"],
    "k_mixed.cu": [],
    "k_mixed_tric.cu": [],
    "coord_api.cu": [],
    "multi.cu": [],
    "peaks.cu": [],
    "noalloc.cu": ["-fmad=false"],
    "bias.cu": ["-fmad=false"],
    "contactmap.cu": ["-fmad=false"],
    "host_setup.cpp": [],
}
HEADERS = ["coord_internal.h", "switch_eval.cuh", "kargs.h", "kernels.cuh", "eval.cuh", "launch.h"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _common():
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "--expt-relaxed-constexpr"]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "coordgpu.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(name: str, extra, verbose: bool, ptxas: bool):
    src = os.path.join(CSRC, name)
    obj = os.path.join(OUT, name + ".o")
    if not _stale(obj, src):
        return obj, ""
    cmd = [nvcc()] + _common() + extra + (["-Xptxas", "-v"] if ptxas else [])
    if name.endswith(".cpp"):
        cmd += ["-x", "cu"]
    cmd += ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (name, " ".join(cmd), p.stderr))
    return obj, p.stderr if (verbose or ptxas) else ""


def build(verbose: bool = False, ptxas: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if force:
        for n in SOURCES:
            o = os.path.join(OUT, n + ".o")
            if os.path.exists(o):
                os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, n, f, verbose, ptxas) for n, f in SOURCES.items()]
        objs = []
        for fu in futs:
            o, log = fu.result()
            objs.append(o)
            if log:
                sys.stderr.write(log)
    relink = not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if relink:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), p.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas="--ptxas" in sys.argv, force="--force" in sys.argv))
