"""Runs the reference build in oracle/_ref (TEST INFRASTRUCTURE ONLY).

The executables come from oracle/build_ref.py: the reference miniAero
sources compiled unmodified against the project's Kokkos stand-in. Each run
takes a miniaero.inp (the reference's input format, kokkos/Options.h:73-100)
and returns the arrays the driver kept: the final conserved state
"solution_n" (ncells, 5), the last stage's "residual", cell centroids and
volumes, and every face set's geometry, connectivity and permutation.

Running the reference needs its source tree (present in the development
container, not on the GPU machine); state_digest() does not.
"""
import hashlib
import os
import subprocess
import tempfile

import numpy as np

from . import build_ref


def available():
    return build_ref.reference_dir() is not None


def input_text(o):
    """miniaero.inp for a reference run: the values Options::read_options_file reads."""
    return "%d\n%r %r %r %r\n%d %d %d\n%d\n%r\n%d\n%d\n%d\n%d\n" % (
        o["problem_type"], float(o["lx"]), float(o["ly"]), float(o["lz"]), float(o.get("angle", 0.0)),
        o["nx"], o["ny"], o["nz"], o["ntimesteps"], float(o["dt"]), int(o.get("output_results", 0)),
        int(o.get("output_frequency", 1 << 30)), int(o.get("second_order_space", 0)), int(o.get("viscous", 0)))


def read_output(path):
    """{label: [array, ...]} in allocation order, from the driver's output file."""
    out = {}
    with open(path, "rb") as f:
        if f.readline() != b"MAREF1\n":
            raise ValueError("not a reference-build output: %s" % path)
        while True:
            head = f.readline()
            if not head:
                break
            parts = head.split()
            label, kind, rank = parts[0].decode(), parts[1].decode(), int(parts[2])
            shape = tuple(int(x) for x in parts[3:3 + rank])
            dtype = np.int32 if kind == "i" else np.float64
            n = int(np.prod(shape)) if shape else 0
            a = np.frombuffer(f.read(n * np.dtype(dtype).itemsize), dtype=dtype).reshape(shape)
            out.setdefault(label, []).append(a)
    return out


def run(inp, variant="miniaero_ref_serial", workdir=None, timeout=3600, env=None):
    """Runs one reference build on a miniaero.inp given as text (or as a dict
    for input_text). Returns (arrays, stdout, results.0 text or None)."""
    exe = build_ref.build([variant])
    if exe is None:
        raise RuntimeError("reference tree not present")
    text = inp if isinstance(inp, str) else input_text(inp)
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        with open(os.path.join(d, "miniaero.inp"), "w") as f:
            f.write(text)
        out = os.path.join(d, "state.bin")
        r = subprocess.run([exe[variant], d, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                           timeout=timeout, env=env)
        if r.returncode != 0:
            raise RuntimeError("reference run failed (%d):\n%s" % (r.returncode, r.stdout[-4000:]))
        arrays = read_output(out)
        res_path = os.path.join(d, "results.0")
        results = open(res_path).read() if os.path.exists(res_path) else None
    return arrays, r.stdout, results


def state_digest(U):
    """SHA-256 of an (ncells, 5) float64 array in C order (the bits, not the values)."""
    U = np.ascontiguousarray(U, dtype="<f8")
    return hashlib.sha256(U.tobytes()).hexdigest()
