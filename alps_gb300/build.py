"""Builds the native library alps_gb300/lib/libalps_gb300.so with nvcc for
sm_103a (GB300).  No GPU is needed to build; the translation units compile in
parallel."""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libalps_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
SOURCES = ["tc_gemm.cu", "batch_solve.cu", "setup_kernels.cu", "disp_kernels.cu", "rel_kernels.cu", "nhds_kernels.cu", "server.cu", "alps_api.cu", "host_tools.cpp", "host_io.cpp"]
HEADERS = ["alps_internal.cuh", "device_math.cuh", "root_finders.h", "root_machine.cuh", "tc_gemm.cuh"]


def _flags(src):
    # host code: no FMA contraction (aarch64 g++ contracts a+b*c by default),
    # so host-side grids and scan steps round like the reference's
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        return ARCH + ["-lineinfo", "-Xptxas", "-O3"] + common
    return ["-x", "c++"] + common


def _compile(src):
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(HERE, "..", "include", "alps_gb300.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [NVCC, "-c", os.path.join(CSRC, src), "-o", obj] + _flags(src)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
