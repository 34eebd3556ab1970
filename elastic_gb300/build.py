"""Builds libelastic_gb300.so in-tree (elastic_gb300/_build/) with nvcc.

One -gencode for sm_103a, translation units compiled in parallel, no cmake.
Usage: python -m elastic_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import fcntl
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libelastic_gb300.so")
SOURCES = ["api.cu", "assemble.cu", "spmv.cu", "krylov.cu", "krylov_ns.cu", "bcsr.cu", "block_pcg.cu", "server.cu", "stress.cu", "loads.cu", "vtk.cu", "partition.cu", "structure.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build elastic_gb300")


def _flags(extra=()):
    return ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
            "-Xcompiler", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles the stale translation units and relinks the library.  Several
    processes may call this at once (test workers): one builds under an
    exclusive lock while the others wait, and every object and the library
    are written to a temporary name and renamed into place, so that no
    process maps a half-written library."""
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(OUT, ".lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        return _build(force, verbose, ptxas_info)


def _build(force: bool, verbose: bool, ptxas_info: bool) -> str:
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "elastic_gb300.h"))
    nv = nvcc()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        if force or ptxas_info or _stale(o, [s, *headers, __file__]):
            extra = ["-Xptxas", "-v"] if ptxas_info and src.endswith(".cu") else []
            if src.endswith(".cpp"):
                cmd = [nv, "-x", "cu", *_flags(extra), "-c", s, "-o", o + ".tmp"]
            else:
                cmd = [nv, *_flags(extra), "-c", s, "-o", o + ".tmp"]
            jobs.append((cmd, o))
    objs = [os.path.join(OUT, s + ".o") for s in SOURCES]

    def run(job):
        cmd, o = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode == 0:
            os.replace(o + ".tmp", o)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or ptxas_info or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [nv, "-shared", *ARCH, "-o", LIB + ".tmp", *objs, "-lcudart_static", "-lrt",
               "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed: " + " ".join(cmd))
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
