"""Builds libmwgpu.so (CUDA kernels for sm_103a + C-ABI + host mirror) in-tree.

Usage: python -m mrcpp_gb300.build   (or mrcpp_gb300.build.build())

Objects go to mrcpp_gb300/_build/, the library to mrcpp_gb300/libmwgpu.so.
Rebuilds only objects older than their sources or headers.  No cmake: one
nvcc per .cu, one g++ per .cpp, run in parallel, then one link.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmwgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libmwgpu")
    return cand


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _headers():
    hs = glob.glob(os.path.join(HERE, "csrc", "**", "*.h"), recursive=True)
    hs += glob.glob(os.path.join(HERE, "csrc", "**", "*.cuh"), recursive=True)
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False):
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include")]
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(HERE, "csrc", "cuda", "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".cu.o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append([nvcc] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + inc +
                        ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(HERE, "csrc", "host", "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src)[:-4] + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unused-function"] + inc +
                        ["-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lcudart", "-lgomp"])
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    with open(os.path.join(BUILD, "ptxas.log"), "w") as fh:
        fh.write("".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
