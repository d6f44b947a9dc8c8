"""Generates tests/golden/reference_build.json: what the reference itself
computes on the four small cases of tests/golden/make_golden.py (the
reference's three serial test inputs and its 32x64x2 flat-plate parallel
input, run on one rank), in both of its reduction builds.

Each case is run through oracle/_ref: the reference's own sources,
unmodified, compiled against the project's Kokkos stand-in, once with
-DATOMICS_FLUX (kokkos/Makefile:17) and once with -DCELL_FLUX (the
gather-sum variant, kokkos/Flux.h:172-178, GreenGauss.h:129,211). Stored per
case and build: SHA-256 of the final conserved state and of the last stage's
residual (ncells x 5 doubles, C order), and per-variable L2 norms. The GPU
tests compare the CUDA path's bits against these digests, and the CPU tests
tie the oracle and the committed oracle fixtures to them, without the
reference tree.

Run in the development container:  python tests/golden/make_reference_digests.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from tests.golden.make_golden import CASES  # noqa: E402

OUT = os.path.join(HERE, "reference_build.json")
BUILDS = {"atomics": "miniaero_ref_serial", "cell_flux": "miniaero_ref_serial_cellflux"}


def inp(case):
    pt, lx, ly, lz, angle, nx, ny, nz, steps, dt, second, visc = CASES[case]
    return dict(problem_type=pt, lx=lx, ly=ly, lz=lz, angle=angle, nx=nx, ny=ny, nz=nz, ntimesteps=steps, dt=dt,
                second_order_space=second, viscous=visc)


def main():
    if not ref.available():
        sys.exit("reference tree not found (set MINIAERO_REFERENCE)")
    out = {"generated_by": "tests/golden/make_reference_digests.py", "cases": {}}
    for case in CASES:
        entry = {"input": inp(case)}
        for build, variant in BUILDS.items():
            arrays, _, _ = ref.run(inp(case), variant=variant)
            U = arrays["solution_n"][0]
            R = arrays["residual"][0]
            entry[build] = {"state_sha256": ref.state_digest(U), "residual_sha256": ref.state_digest(R),
                            "state_l2": [float(np.linalg.norm(U[:, k])) for k in range(5)]}
            print(case, build, entry[build]["state_sha256"][:16], flush=True)
        out["cases"][case] = entry
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
