"""Build recipe of the GB300 QuadRay engine library.

Compiles the CUDA tracer, the C ABI and the C++ host (flattening, engine API,
Python shim) for sm_103a into ``_build/libquadray_gb300.so`` next to this
file.  Numerics flags: device code without FMA contraction and with IEEE
division / square root, host code with ``-ffp-contract=off`` so the host
update phases give the same bits on x86-64 and AArch64.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libquadray_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
DEV_FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-prec-div=true",
             "-prec-sqrt=true", "-ftz=false", "-std=c++17"]
HOST_FLAGS = ["-Xcompiler", "-fPIC,-O2,-ffp-contract=off,-fno-fast-math"]
INCS = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include")]

SOURCES = ["tracer.cu", "tracer_stats.cu", "wavefront.cu", "whitted_wf.cu", "capi.cu", "noalloc.cu",
           "batch.cu",
           "anim.cu", "peak.cu",
           "accel.cpp", "flatten.cpp", "engine.cpp", "pyshim.cpp"]
# sources that textually include another translation unit
INCLUDES = {"tracer_stats.cu": ["tracer.cu"]}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("build step failed: " + " ".join(cmd))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile every translation unit in parallel and link the library."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".h", ".hpp", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "qr_gpu.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        extra = [os.path.join(CSRC, f) for f in INCLUDES.get(src, [])]
        if force or _stale(obj, [path] + headers + extra):
            cmd = [nvcc] + ARCH + DEV_FLAGS + HOST_FLAGS + INCS + \
                  ["-c", path, "-o", obj]
            if src.endswith(".cu"):
                cmd.insert(1, "-Xptxas=-v" if verbose else "-Xptxas=-O3")
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
