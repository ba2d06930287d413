import ctypes
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
EPS_PLAQ_060 = 0.43374  # synthetic gauge recipe: mean plaquette ~0.60


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the library's kernels")


def _cuda_devices() -> int:
    for name in ("libcuda.so.1", "libcuda.so"):
        try:
            cu = ctypes.CDLL(name)
        except OSError:
            continue
        if cu.cuInit(0) != 0:
            return 0
        n = ctypes.c_int()
        if cu.cuDeviceGetCount(ctypes.byref(n)) != 0:
            return 0
        return n.value
    return 0


@pytest.fixture(scope="session")
def orc():
    from oracle.oracle import ORACLE_SO, Oracle, build

    if not os.path.exists(ORACLE_SO):
        build(with_ref=False)
    return Oracle()


@pytest.fixture(scope="session")
def ref():
    from oracle.oracle import Reference

    if not Reference.available():
        pytest.skip("reference library not built here (needs the reference source tree)")
    return Reference()


@pytest.fixture(scope="session")
def refio():
    from oracle.oracle import ReferenceIO

    if not ReferenceIO.available():
        pytest.skip("reference file readers not built here (needs the reference source tree)")
    return ReferenceIO()


@pytest.fixture(scope="session")
def qlib():
    import qcd_gb300
    from qcd_gb300 import build

    if not os.path.exists(qcd_gb300.LIB_PATH):
        build.build()
    return qcd_gb300.lib()


@pytest.fixture(scope="session")
def gpu(qlib):
    if _cuda_devices() < 1:
        pytest.skip("no CUDA device")
    return qlib


@pytest.fixture(scope="session")
def golden():
    out = {}
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            d = np.load(os.path.join(GOLDEN, f))
            out[f[:-4]] = {k: d[k] for k in d.files}
    return out
