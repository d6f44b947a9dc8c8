"""Recipe for oracle/_ref: the reference miniAero sources, unmodified, compiled
against the project's Kokkos stand-in (oracle/kokkos_shim). Test
infrastructure only: the product never links or runs what this builds.

The reference's own build needs Kokkos (kokkos/Makefile:1) and, for its MPI
variant, an MPI library; neither exists here, so this recipe compiles the
sources where they lie (never copying them) with g++ and the stand-in headers
first on the include path. It builds three executables into oracle/_ref/:

  miniaero_ref_serial           -DATOMICS_FLUX, Serial back end: the parity
                                build (the order of the reference's
                                *_Serial golden files)
  miniaero_ref_serial_cellflux  -DCELL_FLUX, Serial back end: the reference's
                                gather-sum variant (kokkos/Flux.h:172-178)
  miniaero_ref_openmp           -DATOMICS_FLUX, OpenMP back end, the
                                reference Makefile's -O3 -g: for timing

The serial builds add -ffp-contract=off (aarch64 g++ contracts a*b+c by
default; x86-64 without -mfma never does), so their arithmetic is the
reference's x86 build's. The OpenMP build keeps the compiler's default.

The reference tree is found at $MINIAERO_REFERENCE (a directory holding the
kokkos/ sources, or that directory itself) or /root/reference/kokkos.
Without it, build() returns None.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(HERE, "kokkos_shim")
DRIVER = os.path.join(HERE, "ref_driver.cpp")
OUT = os.path.join(HERE, "_ref")

# The reference's translation units on the solve path (kokkos/Main.C is
# replaced by ref_driver.cpp; the YAML writer is not on the path).
SOURCES = ["Cell.C", "CopyGhost.C", "ElementTopo.C", "ElementTopoHexa8.C", "Face.C", "MemoryUsage.C",
           "MeshProcessor.C", "Parallel3DMesh.C"]

VARIANTS = {
    "miniaero_ref_serial": ["-O3", "-g", "-DATOMICS_FLUX", "-ffp-contract=off"],
    "miniaero_ref_serial_cellflux": ["-O3", "-g", "-DCELL_FLUX", "-ffp-contract=off"],
    "miniaero_ref_openmp": ["-O3", "-g", "-DATOMICS_FLUX", "-DMINIAERO_SHIM_OPENMP", "-fopenmp"],
}


def reference_dir():
    for cand in (os.environ.get("MINIAERO_REFERENCE"), "/root/reference/kokkos"):
        if cand and os.path.isfile(os.path.join(cand, "TimeSolverExplicitRK4.h")):
            return cand
        if cand and os.path.isfile(os.path.join(cand, "kokkos", "TimeSolverExplicitRK4.h")):
            return os.path.join(cand, "kokkos")
    return None


def exe(variant):
    return os.path.join(OUT, variant)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(variants=None, jobs=None):
    """Compiles the requested variants (default: all) if stale. Returns
    {variant: executable path}, or None when the reference tree is absent."""
    ref = reference_dir()
    if ref is None:
        return None
    variants = list(variants or VARIANTS)
    shim_files = [os.path.join(dp, f) for dp, _, fs in os.walk(SHIM) for f in fs]
    ref_files = [os.path.join(ref, f) for f in os.listdir(ref) if f.endswith((".h", ".C"))]
    deps = shim_files + ref_files + [DRIVER, os.path.abspath(__file__)]
    compile_jobs, links = [], []
    for v in variants:
        if not _newer(exe(v), deps):
            continue
        objdir = os.path.join(OUT, "obj_" + v)
        os.makedirs(objdir, exist_ok=True)
        flags = ["g++", "-std=c++14", "-w"] + VARIANTS[v] + ["-I" + SHIM, "-I" + ref]
        objs = []
        for src in SOURCES + [DRIVER]:
            path = src if os.path.isabs(src) else os.path.join(ref, src)
            obj = os.path.join(objdir, os.path.basename(path).rsplit(".", 1)[0] + ".o")
            compile_jobs.append(flags + ["-x", "c++", "-c", path, "-o", obj])
            objs.append(obj)
        links.append(["g++"] + VARIANTS[v] + objs + ["-o", exe(v)])
    if compile_jobs:
        with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
            list(ex.map(_run, compile_jobs))
        for cmd in links:
            _run(cmd)
    return {v: exe(v) for v in variants}


if __name__ == "__main__":
    res = build(sys.argv[1:] or None)
    if res is None:
        print("reference tree not found; nothing built")
    else:
        for v, p in res.items():
            print(v, p)
