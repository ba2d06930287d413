"""Multi-RHS tensor-core operator: every RHS slot against the FP64 oracle.

Storage is FP16 with a per-(site, RHS) norm; the products run in FP32 (SIMT
kernel) or as TF32 on the tensor cores with FP32 accumulation. The bar is the
FP16 single-RHS one (4e-3 relative per RHS), for every kernel variant."""
import numpy as np
import pytest

import qcd_gb300 as q
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
TOL = 4e-3


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(params=[-1, 1, 128, 129], ids=["tuned", "tensor", "simt128", "simt128x2"])
def variant(request, gpu):
    q.set_mrhs_variant(request.param)
    yield request.param
    q.set_mrhs_variant(-1)


@pytest.mark.parametrize("nrhs,nact", [(5, 5), (16, 16), (20, 17), (48, 48)])
@pytest.mark.parametrize("op", [q.OP_D, q.OP_DDAG])
def test_mrhs_operator_each_rhs_matches_oracle(gpu, orc, variant, nrhs, nact, op):
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
    for o in (g, mi, mo, f):
        o.close()
