"""The float-float FP64 operator (FP64 storage, FP32-pipe arithmetic with
FP64 spin projections) against the CPU oracle at <= 1e-13 relative per-site
norm: D, D^+ and Q with twisted mass, boundary phases in two directions and
a lattice whose last 128-site block is partial; its even/odd form inside an
even/odd solve, checked by the FP64 true residual."""
import numpy as np
import pytest

import qcd_gb300 as q
from oracle.oracle import site_rel_err
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
TOL64 = 1e-13


@pytest.mark.parametrize("L", [(8, 6, 4, 10), (4, 4, 4, 4), (16, 8, 8, 8)])
def test_float_float_operator_vs_oracle(gpu, orc, L):
    th = (np.pi, 0.0, 0.2, 0.0)
    u = orc.gauge_synthetic(L, 31, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 32)
    g = q.Gauge(L, th).load(u)
    fin, fout = q.Field(L).load(v), q.Field(L)
    for op, o in ((q.OP_D, "D"), (q.OP_DDAG, "Ddag"), (q.OP_Q, "Q")):
        q.dslash(fout, fin, g, 0.15, 0.07, op, q.ARITH_DF64)
        assert site_rel_err(fout.store(), orc.dslash(v, u, L, th, kappa=0.15, tm=0.07, op=o)) <= TOL64, o
    for f in (g, fin, fout):
        f.close()


def test_float_float_even_odd_solve(gpu, orc):
    # the even/odd solver's FP64 restarts, source preparation and
    # reconstruction run the float-float even/odd kernels
    L = (8, 8, 8, 8)
    th = (np.pi, 0.0, 0.0, 0.3)
    u = orc.gauge_synthetic(L, 41, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 42)
    g = q.Gauge(L, th).load(u)
    b, x = q.Field(L).load(v), q.Field(L)
    p = q.solve(x, b, g, 0.15, 0.03, solver=q.SOLVER_CGNR_EO, inner_prec=q.F32, tol=1e-10)
    assert p.status == 0
    assert orc.true_residual(x.store(), v, u, L, th, 0.15, 0.03) <= 1e-10
    for f in (g, b, x):
        f.close()
