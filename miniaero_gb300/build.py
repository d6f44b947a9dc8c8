"""Build recipe for libminiaero_gpu.so, the miniaero CLI and the oracle.

Compiles every translation unit in parallel with nvcc (sm_103a) or g++, links
in-tree under miniaero_gb300/_build/ (and oracle/_build/ for the oracle).
Host floating-point code is built with -ffp-contract=off and the FP64 device
code with --fmad=false: the plain form reproduces the reference's serial
arithmetic bit for bit only without contracted multiply-adds.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

LIB = os.path.join(BUILD, "libminiaero_gpu.so")
CLI = os.path.join(BUILD, "miniaero")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libminiaero_oracle.so")
# The same oracle source built the way the reference's Makefile builds its
# code (-O3 -g, the compiler's default contraction of a*b+c, which aarch64 g++
# turns into fused multiply-adds): the CPU timing baseline only. Its sums are
# not the reference's serial bits, so parity checks use ORACLE_LIB.
ORACLE_TIMING_LIB = os.path.join(ORACLE_BUILD, "libminiaero_oracle_timing.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off"] + ARCH
HOST_CXX = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]

# (source, extra flags)
DEVICE_SOURCES = [
    ("device/kernels_fp64.cu", ["--fmad=false"]),
    # The opt-in contracted FP64 form (MA_PREC_FP64_FMA).
    ("device/kernels_fp64_fma.cu", ["--fmad=true"]),
    # FP32 division and square root as the full-range approximations (within
    # 2 ulp): the IEEE forms' slow-path branches cost the mixed sweep 16 % and
    # the mixed flux 6 %, and the mixed form keeps no reference bits.
    ("device/kernels_mixed.cu", ["--fmad=false", "-prec-div=false", "-prec-sqrt=false"]),
    ("device/ops.cu", ["--fmad=false"]),
    ("device/solver.cu", ["--fmad=false"]),
    ("device/batch.cu", ["--fmad=false"]),
    ("device/noalloc.cu", ["--fmad=false"]),
    # Mesh geometry on the device, bit-identical to the host generator.
    ("device/geometry.cu", ["--fmad=false"]),
]
HOST_SOURCES = ["host/mesh.cpp", "host/options.cpp", "host/host_api.cpp", "host/server.cpp", "host/checkpoint.cpp"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _obj(src):
    return os.path.join(BUILD, src.replace("/", "_").rsplit(".", 1)[0] + ".o")


def build(verbose=False, ptxas_info=False):
    """Compiles the library, the CLI and the oracle. Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    nvcc = _nvcc()
    cuda_include = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")  # NVTX headers
    jobs = []
    for src, extra in DEVICE_SOURCES:
        cmd = [nvcc] + NVCC_COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", _obj(src)]
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        jobs.append(cmd)
    for src in HOST_SOURCES:
        jobs.append(HOST_CXX + ["-I" + cuda_include, "-c", os.path.join(CSRC, src), "-o", _obj(src)])
    jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-fopenmp", "-shared",
                 os.path.join(ORACLE, "miniaero_oracle.c"), "-o", ORACLE_LIB, "-lm"])
    jobs.append(["gcc", "-O3", "-g", "-std=c11", "-fPIC", "-fopenmp", "-shared",
                 os.path.join(ORACLE, "miniaero_oracle.c"), "-o", ORACLE_TIMING_LIB, "-lm"])
    outputs = []
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for out in ex.map(lambda c: _run(c, verbose), jobs):
            outputs.append(out)
    objs = [_obj(s) for s, _ in DEVICE_SOURCES] + [_obj(s) for s in HOST_SOURCES]
    _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static", "-lpthread", "-ldl"], verbose)
    _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(CSRC, "cli", "main.cpp"),
          "-o", CLI, "-L" + BUILD, "-lminiaero_gpu", "-Wl,-rpath,$ORIGIN"], verbose)
    if ptxas_info:
        return LIB, "\n".join(outputs)
    return LIB


if __name__ == "__main__":
    info = "--ptxas" in sys.argv
    res = build(verbose="-v" in sys.argv, ptxas_info=info)
    if info:
        print(res[1])
    print("built", LIB)
