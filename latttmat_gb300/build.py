"""Build liblatttmat_gb300.so (CUDA, sm_103a) and the tmat and dumpconfig CLIs in-tree.

nvcc compiles each translation unit in parallel with
``-gencode arch=compute_103a,code=sm_103a``; objects go to
``latttmat_gb300/_build/`` and the shared library to
``latttmat_gb300/liblatttmat_gb300.so``.  No torch or cmake involved.
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
LIB = os.path.join(HERE, "liblatttmat_gb300.so")
CLI = os.path.join(HERE, "tmat")
DUMP_CLI = os.path.join(HERE, "dumpconfig")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "latttmat.h"))
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, extra_flags=None) -> str:
    """Compile every .cu under csrc/ and link the shared library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])
    headers = _headers()
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    if jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"])
    host_dir = os.path.join(HERE, "host")
    if os.path.isdir(host_dir):
        host_hdrs = [os.path.join(host_dir, f) for f in os.listdir(host_dir) if f.endswith(".hpp")]
        for exe, main in ((CLI, "tmat_main.cpp"), (DUMP_CLI, "dumpconfig_main.cpp")):
            src = os.path.join(host_dir, main)
            if os.path.exists(src) and _stale(exe, [src, LIB] + host_hdrs):
                _run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", host_dir,
                      src, "-o", exe, "-L", HERE, "-llatttmat_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
