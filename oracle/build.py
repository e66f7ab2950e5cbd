"""Build the test oracle (TEST INFRASTRUCTURE ONLY).

``build_oracle()`` compiles the CPU restatement ``qr_oracle.c`` into
``oracle/_build/libqr_oracle.so`` (plain C, ``-ffp-contract=off``, no
fast-math).  ``build_ref()`` compiles the reference engine's own renderer
from its sources with ``oracle/Makefile`` into ``oracle/_ref/`` when the
reference tree is available (the golden-fixture generator uses it).

``build_oracle_gpu()`` compiles the same source in double for the device
(``qr_oracle_gpu.cu``: the FP64 path-tracer oracle on the GPU).

``load_oracle()`` and ``load_oracle_gpu()`` return ctypes handles; only
tests, the smoke check and the CPU-baseline leg of bench.py call them.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libqr_oracle.so")
LIB64 = os.path.join(OUT, "libqr_oracle64.so")     # QR_ORACLE_FP64 build
# the reference checkout: QR_REFERENCE, else /root/reference (read-only);
# where neither holds the reference's sources its build is skipped
REF_DIR = os.environ.get("QR_REFERENCE") or "/root/reference"
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")


def build_oracle(fp64=False):
    """Compile qr_oracle.c in float (the checker, the CPU baseline) or, with
    fp64, in double (the FP64 path-tracer oracle)."""
    os.makedirs(OUT, exist_ok=True)
    lib = LIB64 if fp64 else LIB
    src = os.path.join(HERE, "qr_oracle.c")
    deps = [src, os.path.join(HERE, "qr_oracle.h"), os.path.join(ROOT, "include", "qr_gpu.h")]
    if os.path.exists(lib) and all(os.path.getmtime(d) <= os.path.getmtime(lib) for d in deps):
        return lib
    cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-fPIC", "-shared",
           "-ffp-contract=off", "-fno-fast-math", "-I" + HERE,
           "-I" + os.path.join(ROOT, "include")] + (["-DQR_ORACLE_FP64"] if fp64 else []) + \
          [src, "-lm", "-o", lib]
    subprocess.run(cmd, check=True)
    return lib


LIBGPU = os.path.join(OUT, "libqr_oracle_gpu.so")   # FP64 oracle on the GPU


def build_oracle_gpu():
    """Compile qr_oracle_gpu.cu (qr_oracle.c in double, for the device) for
    sm_103a; nvcc cross-compiles it without a GPU"""
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "qr_oracle_gpu.cu")
    deps = [src, os.path.join(HERE, "qr_oracle.c"), os.path.join(HERE, "qr_oracle.h"),
            os.path.join(ROOT, "include", "qr_gpu.h")]
    if os.path.exists(LIBGPU) and all(os.path.getmtime(d) <= os.path.getmtime(LIBGPU)
                                      for d in deps):
        return LIBGPU
    nvcc = os.environ.get("NVCC") or (
        "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
           "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I" + HERE,
           "-I" + os.path.join(ROOT, "include"), "-shared", src, "-o", LIBGPU]
    subprocess.run(cmd, check=True)
    return LIBGPU


def load_oracle_gpu():
    L = ctypes.CDLL(build_oracle_gpu())
    L.qr_oracle_pt_gpu.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
    return L


def build_ref():
    """Build oracle/_ref/ref_driver from the reference sources, if present."""
    if not os.path.isdir(os.path.join(REF_DIR, "core", "engine")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_DIR], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_DRIVER


def load_oracle(fp64=False):
    L = ctypes.CDLL(build_oracle(fp64))
    L.qr_oracle_render.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_uint64)]
    L.qr_oracle_pt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_uint64)]
    return L
