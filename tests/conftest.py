import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: longer CPU test")


def _sources_newer_than(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for base in ("miniaero_gb300/csrc", "oracle", "include"):
        for dp, _, files in os.walk(os.path.join(ROOT, base)):
            if "_build" in dp:
                continue
            for f in files:
                if f.endswith((".cu", ".cuh", ".cpp", ".hpp", ".h", ".c")):
                    if os.path.getmtime(os.path.join(dp, f)) > t:
                        return True
    return False


@pytest.fixture(scope="session", autouse=True)
def built():
    """Builds the library and the oracle once if they are missing or stale."""
    from miniaero_gb300 import build as b
    if any(_sources_newer_than(t) for t in (b.LIB, b.ORACLE_LIB, b.ORACLE_TIMING_LIB)):
        b.build()
    return True


@pytest.fixture(scope="session")
def reference_dir():
    """The reference's kokkos/ source tree: $MINIAERO_REFERENCE, else where the
    oracle's reference-build recipe looks for it. Tests that read it skip where
    it is absent (the GPU machine)."""
    from oracle import build_ref
    d = build_ref.reference_dir()
    if d is None:
        pytest.skip("reference tree not present (set MINIAERO_REFERENCE)")
    return d


@pytest.fixture(scope="session")
def has_gpu():
    import miniaero_gb300 as ma
    if ma.device_count() < 1:
        pytest.fail("GPU test needs a CUDA device")
    return True
