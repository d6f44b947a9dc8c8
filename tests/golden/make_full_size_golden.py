"""Generates tests/golden/full_size.json: SHA-256 digests and per-variable L2
norms of the FP64 conserved state after a few RK4 steps on the full-size
meshes, for the GPU tests to compare bit for bit.

Four cases, each at dt from CFL 0.5 on its initial state (computed here once
and stored, so every side runs the same dt):
  * reference_sod_2nd_viscous_256x128x128: the reference's own Sod problem
    (its initial state, Sutherland viscosity, Venkatakrishnan limiter) on the
    Sod benchmark's 256x128x128 mesh of 1.0x0.5x0.5. Digest of the REFERENCE
    itself: its unmodified sources compiled against the Kokkos stand-in
    (oracle/_ref/miniaero_ref_serial); the oracle is checked to give the same
    bits.
  * reference_flat_plate_2nd_viscous_512x128x128: the reference's flat-plate
    problem (its Mach ~2.5 inflow, Venkatakrishnan) on the flat-plate
    benchmark's 512x128x128 mesh of 2.0x0.5x0.5, again from the reference.
  * sod_2nd_viscous_256x128x128 and flat_plate_vanalbada_512x128x128: the
    benchmark configurations exactly (Sod rho/p = 1/1 | 0.125/0.1, constant
    viscosity 1.8e-5 with Pr 0.72; flat plate at Mach 0.3, p = 1e5, T = 300 K
    with the Van Albada limiter). The reference cannot express these inputs,
    so their digests come from the serial oracle.

Run in the development container, where the reference tree is present:
    python tests/golden/make_full_size_golden.py [--steps N] [--skip-oracle-check] [--only NAME ...]
Takes tens of minutes and up to ~45 GB of host memory (the reference build
holds about 4.5 KB per cell on the 8.4 M-cell mesh).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import miniaero_gb300 as ma  # noqa: E402
import oracle  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.join(HERE, "full_size.json")

REFERENCE_CASES = {
    "reference_sod_2nd_viscous_256x128x128": dict(problem_type=0, lx=1.0, ly=0.5, lz=0.5, nx=256, ny=128,
                                                  nz=128, second_order_space=1, viscous=1),
    "reference_flat_plate_2nd_viscous_512x128x128": dict(problem_type=1, lx=2.0, ly=0.5, lz=0.5, nx=512, ny=128,
                                                         nz=128, second_order_space=1, viscous=1),
}
ORACLE_CASES = ["sod_2nd_viscous_256x128x128", "flat_plate_vanalbada_512x128x128"]


def options_dict(o):
    return {name: getattr(o, name) for name, _ in ma._lib.ma_options._fields_}


def summary(U):
    return {"sha256": ref.state_digest(U), "l2": [float(np.linalg.norm(U[:, k])) for k in range(5)]}


def log(*a):
    print(time.strftime("%H:%M:%S"), *a, flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--skip-oracle-check", action="store_true")
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    if not ref.available():
        sys.exit("reference tree not found (set MINIAERO_REFERENCE)")
    data = {"generated_by": "tests/golden/make_full_size_golden.py", "cases": {}}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data["cases"] = json.load(f).get("cases", {})
    for name in list(REFERENCE_CASES) + ORACLE_CASES:
        if args.only and name not in args.only:
            continue
        if name in REFERENCE_CASES:
            o = ma.Options(**REFERENCE_CASES[name])
        else:
            o = bench.make_options(ma, name, "fp64")
        log(name, "mesh")
        md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
        U0 = ma.initial_state(md, o)
        dt = bench.cfl_dt_host(md, U0, 0.5)
        o.cfl = 0.0
        o.dt = dt
        o.ntimesteps = args.steps
        case = {"source": None, "options": options_dict(o), "cells": md.ncells, "steps": args.steps, "dt": dt}
        if name in REFERENCE_CASES:
            inp = dict(REFERENCE_CASES[name], dt=dt, ntimesteps=args.steps)
            log(name, "reference run")
            t0 = time.time()
            arrays, _, _ = ref.run(inp)
            R = np.array(arrays["solution_n"][0])
            del arrays
            case.update(source="reference build (oracle/_ref/miniaero_ref_serial)", reference_s=time.time() - t0)
            case.update(summary(R))
            if not args.skip_oracle_check:
                log(name, "oracle run")
                U = oracle.solve(md, o, U0)
                case["oracle_bit_equal"] = bool(np.array_equal(U.view(np.uint64), R.view(np.uint64)))
                if not case["oracle_bit_equal"]:
                    raise SystemExit("%s: oracle differs from the reference build" % name)
        else:
            log(name, "oracle run")
            t0 = time.time()
            U = oracle.solve(md, o, U0)
            case.update(source="serial oracle (oracle/miniaero_oracle.c)", oracle_s=time.time() - t0)
            case.update(summary(U))
        data["cases"][name] = case
        log(name, case["sha256"])
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1)
        del md, U0


if __name__ == "__main__":
    main()
