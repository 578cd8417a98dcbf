"""Build recipe of the engine's shared library (nvcc, sm_103a only).

    python -m hpdbscan_gb300.build        # -> hpdbscan_gb300/libhpdbscan_gb300.so

Every translation unit under csrc/ is compiled in parallel and linked into one
shared library that exports the C ABI of include/hpdbscan_gb300.h.  Host code is
compiled with -ffp-contract=off so that the host-side grid arithmetic rounds every
operation exactly as written on both x86-64 and aarch64 hosts.
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhpdbscan_gb300.so")
CLI = os.path.join(HERE, "hpdbscan")  # command line tool (csrc/hpdbscan_cli.cpp)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def sources():
    """Every translation unit of the library: the CUDA sources and the host-only C++ ones."""
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu") or (f.endswith(".cpp") and f != "hpdbscan_cli.cpp"))


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "hpdbscan_gb300.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.splitext(os.path.basename(s))[0] + ".o") for s in srcs]
    jobs = []
    for s, o in zip(srcs, objs):
        if _stale(o, s) or ptxas_info:
            cmd = [cc] + _flags() + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", s, "-o", o]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose or ptxas_info or r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        link = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "hpdbscan_cli.cpp")
    if not os.path.exists(CLI) or os.path.getmtime(cli_src) > os.path.getmtime(CLI) or \
            os.path.getmtime(LIB) > os.path.getmtime(CLI):
        cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), cli_src, "-o", CLI,
               "-L", HERE, "-lhpdbscan_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("CLI build failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
