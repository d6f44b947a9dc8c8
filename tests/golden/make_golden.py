"""Generates tests/golden/reference_cases.npz: the final conserved state of the
reference's three serial test cases (kokkos/tests/{3D_Sod,Ramp,FlatPlate}_Serial/
miniaero.inp parameters) computed by the serial oracle, and SHA-256 digests of
the host mesh arrays (connectivity, permutations, geometry).

The oracle itself is pinned to the reference's results.gold and
results.<rank>.gold files by tests/test_oracle_gold.py; these fixtures carry that pin to machines without
the reference tree (the GPU tests compare against them bit for bit).

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import miniaero_gb300 as ma  # noqa: E402
import oracle  # noqa: E402

# (problem_type, lx, ly, lz, angle, nx, ny, nz, steps, dt, second_order, viscous)
CASES = {
    "sod_serial": (0, 0.3048, 1.0, 1.0, 0.0, 128, 4, 4, 100, 2e-6, 0, 0),
    "ramp_serial": (2, 2.0, 2.0, 1.0, 30.0, 64, 32, 2, 400, 1e-5, 1, 0),
    "flatplate_serial": (1, 2.0, 0.002, 1.0, 0.0, 16, 32, 2, 400, 3e-8, 1, 1),
    "flatplate_parallel": (1, 2.0, 0.002, 1.0, 0.0, 32, 64, 2, 400, 1e-8, 1, 1),
}


def options(case):
    pt, lx, ly, lz, angle, nx, ny, nz, steps, dt, second, visc = CASES[case]
    return ma.Options(problem_type=pt, lx=lx, ly=ly, lz=lz, angle=angle, nx=nx, ny=ny, nz=nz, ntimesteps=steps,
                      dt=dt, second_order_space=second, viscous=visc)


def mesh_digest(md):
    h = hashlib.sha256()
    for fs in [md.internal] + md.bc:
        for a in (fs.conn, fs.permutation, fs.coords, fs.normal, fs.tangent, fs.binormal):
            h.update(np.ascontiguousarray(a).tobytes())
    h.update(md.cell_coords.tobytes())
    h.update(md.cell_volumes.tobytes())
    return h.hexdigest()


def main():
    out = {}
    for case in CASES:
        o = options(case)
        md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
        U = oracle.solve(md, o, ma.initial_state(md, o))
        out[case + "_U"] = U
        out[case + "_mesh_sha256"] = np.array(mesh_digest(md))
        print(case, md.ncells, mesh_digest(md)[:16])
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_cases.npz"), **out)


if __name__ == "__main__":
    main()
