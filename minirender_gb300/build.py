"""Builds the in-tree shared library minirender_gb300/_lib/libminirender_gpu.so
from csrc/ with nvcc for sm_103a (three translation units compiled in
parallel, then linked; CUDA runtime linked statically)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libminirender_gpu.so")
SOURCES = ["kernels.cu", "capi.cpp", "host_math.cpp", "noalloc.cu", "server.cpp", "loaders.cpp"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false / IEEE division and sqrt / no flush-to-zero on the device, and
# -ffp-contract=off on the host: the operation order of the reference CPU
# renderer is reproduced exactly (coverage and depth are compared bit for bit).
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-fmad=false",
           "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
           "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden,-O2"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [
        os.path.join(HERE, "..", "include", "minirender_gpu.h"), __file__]
    if not force and _newer(LIB, deps):
        return LIB
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = [nv] + ARCH + NVFLAGS + ["-c", os.path.join(SRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose:
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
