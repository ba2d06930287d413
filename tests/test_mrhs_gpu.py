"""Multi-RHS operator: every RHS slot against the FP64 oracle.

Storage is FP16 with a per-(site, RHS) norm; the products run in FP32 (SIMT
kernel), as FP16 tcgen05 MMAs with FP32 accumulation in tensor memory, or as
TF32 mma.sync with FP32 accumulation. The bar is the FP16 single-RHS one
(4e-3 relative per RHS), for every kernel variant."""
import ctypes as C

import numpy as np
import pytest

import qcd_gb300 as q
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
TOL = 4e-3


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(params=[-1, 1, 2, 128, 129], ids=["tuned", "mma_sync", "tcgen05", "simt128", "simt128x2"])
def variant(request, gpu):
    q.set_mrhs_variant(request.param)
    yield request.param
    q.set_mrhs_variant(-1)


def tc_timeouts():
    n = C.c_uint(0)
    assert q.lib().qcdgpu_mrhs_tc_timeouts(C.byref(n)) == 0
    return n.value


@pytest.mark.parametrize("nrhs,nact", [(5, 5), (16, 16), (20, 17), (32, 23), (48, 48)])
@pytest.mark.parametrize("op", [q.OP_D, q.OP_DDAG])
def test_mrhs_operator_each_rhs_matches_oracle(gpu, orc, variant, nrhs, nact, op):
    if variant == 2 and nrhs % 16:
        pytest.skip("the tcgen05 kernel takes slot counts that are multiples of 16")
    L = (8, 4, 6, 4)
    th = (np.pi, 0.0, 0.3, 0.0)
    u = orc.gauge_synthetic(L, 41, EPS_PLAQ_060)
    g = q.Gauge(L, th).load(u)
    mi, mo = q.MField(L, nrhs), q.MField(L, nrhs)
    srcs = []
    f = q.Field(L)
    for r in range(nrhs):
        v = orc.gaussian_spinor(L, 100 + r) * (10.0 ** (r % 5 - 2))  # RHS of very different scales
        srcs.append(v)
        mi.set(r, f.load(v))
    q.dslash_mrhs(mo, mi, g, 0.15, 0.05, op, nact)
    name = "D" if op == q.OP_D else "Ddag"
    for r in range(nact):
        ref = orc.dslash(srcs[r], u, L, th, kappa=0.15, tm=0.05, op=name)
        assert rel(mo.get(r, f).store(), ref) <= TOL, r
    assert tc_timeouts() == 0
    for o in (g, mi, mo, f):
        o.close()


def test_tcgen05_variant_rejects_slot_counts_it_cannot_tile(gpu, orc):
    L = (8, 4, 6, 4)
    g = q.Gauge(L, (0.0, 0.0, 0.0, 0.0)).load(orc.gauge_synthetic(L, 42, EPS_PLAQ_060))
    mi, mo = q.MField(L, 20), q.MField(L, 20)
    q.set_mrhs_variant(2)
    try:
        with pytest.raises(q.QcdGpuError):
            q.dslash_mrhs(mo, mi, g, 0.15, 0.0, q.OP_D, 20)
    finally:
        q.set_mrhs_variant(-1)
        for o in (g, mi, mo):
            o.close()


def test_tcgen05_bounded_wait_runs_out_and_is_reported(gpu, orc):
    """the test hook issues no MMA, so every wait for the accumulator runs out
    (4096 polls): the launch abandons its work, qcdgpu_sync and the next apply
    report the failure, and after a reset the kernel is exact again"""
    L = (8, 4, 6, 4)
    th = (np.pi, 0.0, 0.0, 0.0)
    u = orc.gauge_synthetic(L, 43, EPS_PLAQ_060)
    g = q.Gauge(L, th).load(u)
    mi, mo, f = q.MField(L, 16), q.MField(L, 16), q.Field(L)
    srcs = [orc.gaussian_spinor(L, 200 + r) for r in range(16)]
    for r in range(16):
        mi.set(r, f.load(srcs[r]))
    lib = q.lib()
    q.set_mrhs_variant(2)
    try:
        assert lib.qcdgpu_mrhs_tc_test_hook(1, 4096) == 0
        q.dslash_mrhs(mo, mi, g, 0.15, 0.0, q.OP_D, 16)  # the launch itself is accepted
        assert lib.qcdgpu_sync() == 1
        assert "bounded wait" in lib.qcdgpu_last_error().decode()
        assert tc_timeouts() > 0
        with pytest.raises(q.QcdGpuError):  # refused until the state is cleared
            q.dslash_mrhs(mo, mi, g, 0.15, 0.0, q.OP_D, 16)
    finally:
        lib.qcdgpu_mrhs_tc_test_hook(0, 0)
        assert lib.qcdgpu_mrhs_tc_reset() == 0
    try:
        assert tc_timeouts() == 0
        q.dslash_mrhs(mo, mi, g, 0.15, 0.0, q.OP_D, 16)
        assert lib.qcdgpu_sync() == 0
        for r in (0, 15):
            assert rel(mo.get(r, f).store(), orc.dslash(srcs[r], u, L, th, kappa=0.15)) <= TOL
    finally:
        q.set_mrhs_variant(-1)
        for o in (g, mi, mo, f):
            o.close()
