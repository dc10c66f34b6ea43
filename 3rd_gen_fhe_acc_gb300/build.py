"""Builds libfheacc.so in this directory: the CUDA kernels for sm_103a and the
C++ host runtime, compiled in parallel and linked into one shared library.

    python -m build            (from this directory), or
    import build; build.build_library()
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfheacc.so")

CUDA_SOURCES = ["api.cu", "bootstrap32.cu", "blind_rotate32.cu", "lwe_ks.cu", "probe.cu", "noalloc.cu", "server.cu", "bootstrap64.cu", "expand.cu", "graph.cu", "psi.cu"]
HOST_SOURCES = ["host/params.cpp", "host/keygen.cpp", "host/container.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    return r.stdout


def _obj(src):
    return os.path.join(BUILD, src.replace("/", "_") + ".o")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(ROOT, "include", "fheacc.h")]
    for d, _, fs in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in fs if f.endswith((".cuh", ".hpp", ".h", ".inc"))]
    return hs


def build_library(verbose=False, ptxas_info=False):
    """Compile (when out of date) and link libfheacc.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    hdrs = _headers()
    jobs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        out = _obj(s)
        if ptxas_info or _stale(out, [src] + hdrs):
            cmd = [_nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                      "-c", src, "-o", out] + inc
            if ptxas_info:
                cmd.append("-Xptxas=-v")
            jobs.append(cmd)
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, s)
        out = _obj(s)
        if _stale(out, [src] + hdrs):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-c", src, "-o", out] + inc)
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    objs = [_obj(s) for s in CUDA_SOURCES + HOST_SOURCES]
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


if __name__ == "__main__":
    build_library(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
