"""Builds satsuma2_gb300/libsatsuma2_gb300.so (and the slave executable) for
sm_103a with nvcc, in tree.  Translation units compile in parallel; the
result is reused while no source is newer than it.

    python -m satsuma2_gb300.build [--force]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsatsuma2_gb300.so")
SLAVE = os.path.join(HERE, "satsuma2_slave")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off on the host: the tables the host builds in double (entropy
# terms, probability table) must round exactly as the reference's x86-64 build.
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 "-I", INCLUDE, "-I", CSRC]
LIB_SOURCES = ["xc_corr.cu", "xc_scan.cu", "xc_runtime.cu", "xc_server.cu", "xc_noalloc.cu", "xc_tune.cu"]
SLAVE_SOURCES = ["slave_main.cpp"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _compile(src, extra=()):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if _newer(obj, [src] + _headers()):
        cmd = [NVCC] + COMMON + list(extra) + ["-c", src, "-o", obj]
        subprocess.check_call(cmd)
    return obj


def build(force=False, verbose=False):
    """Compiles the library (and the slave when its source exists); returns the .so path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in LIB_SOURCES]
    deps = srcs + _headers()
    slave_srcs = [os.path.join(CSRC, s) for s in SLAVE_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if force or _newer(LIB, deps):
        if force:
            for f in os.listdir(BUILD):
                os.remove(os.path.join(BUILD, f))
        extra = ["-Xptxas", "-v"] if verbose else []
        with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
            objs = list(ex.map(lambda s: _compile(s, extra), srcs))
        tmp = LIB + ".tmp.%d" % os.getpid()
        subprocess.check_call([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    if slave_srcs and (force or _newer(SLAVE, slave_srcs + deps)):
        objs = [_compile(os.path.join(CSRC, s)) for s in LIB_SOURCES]
        sobj = [_compile(s) for s in slave_srcs]
        tmp = SLAVE + ".tmp.%d" % os.getpid()
        subprocess.check_call([NVCC] + ARCH + ["-o", tmp] + sobj + objs + ["-lpthread"])
        os.replace(tmp, SLAVE)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
