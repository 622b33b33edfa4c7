"""Builds libcppimpact_gb300.so in-tree for sm_103a (no cmake, a few seconds per file).

    python -m cppimpact_gb300.build        # or build() from Python

Host translation units are compiled with g++, the CUDA one with nvcc
``-gencode arch=compute_103a,code=sm_103a -lineinfo``, all in parallel, then linked
with nvcc into ``cppimpact_gb300/libcppimpact_gb300.so``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcppimpact_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["ci_plan.cpp", "ci_inp.cpp"]
CUDA_SOURCES = ["ci_solver.cu", "ci_batch.cu", "ci_gemm.cu", "ci_mlp.cu", "ci_noalloc.cu"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_nvcc: list[str] | None = None, out: str | None = None,
          build_dir: str | None = None) -> str:
    """Compile and link; ``extra_nvcc`` flags (e.g. -D options) go to every CUDA unit,
    ``out`` / ``build_dir`` place a differently configured library elsewhere."""
    lib_path = out or LIB
    bdir = build_dir or BUILD
    os.makedirs(bdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "cppimpact_gb300.h"))
    jobs, objs = [], []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-c", s, "-o", o])
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", *(extra_nvcc or []), "-c", s, "-o", o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for j in jobs]
    failed = False
    for j, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(" ".join(j) + "\n" + (out or ""))
        failed |= p.returncode != 0
    if failed:
        raise RuntimeError("libcppimpact_gb300 build failed")
    if jobs or not os.path.exists(lib_path):
        link = [_nvcc(), *ARCH, "-shared", "-o", lib_path, *objs, "-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return lib_path


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("-v", action="store_true")
    ap.add_argument("-D", action="append", default=[], help="preprocessor define for CUDA units")
    ap.add_argument("--out", default=None, help="library path (default: in-tree)")
    ap.add_argument("--build-dir", default=None)
    a = ap.parse_args()
    print(build(verbose=a.v, extra_nvcc=[f"-D{d}" for d in a.D], out=a.out, build_dir=a.build_dir))
