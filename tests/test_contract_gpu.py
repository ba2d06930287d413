"""Proton two-point function on GPU-resident propagators against the oracle
(FP64, 1e-12 relative) and against twop.c's own output (the golden fixtures,
bounded by its 7 printed digits), with and without sink smearing; and the
whole chain -- twelve point-source solves per flavour, then the contraction
-- without leaving the GPU."""
import numpy as np
import pytest

import qcd_gb300 as q
from tests.conftest import EPS_PLAQ_060
from tests.golden.make_golden import TWOP_MOMS, twop_inputs

pytestmark = pytest.mark.gpu
TH = (np.pi, 0.0, 0.0, 0.0)


@pytest.mark.parametrize("case", ["twop_L8442", "twop_L8442_smeared"])
def test_twop_matches_oracle_and_reference(gpu, orc, golden, case):
    g = golden[case]
    L = tuple(int(x) for x in g["L"])
    xsrc = tuple(int(x) for x in g["xsrc"])
    t0, t1, nsm, nape = int(g["t0"]), int(g["t1"]), int(g["nsmear"]), int(g["nape"])
    u, cu, cd, prop = twop_inputs(orc, L, int(g["seed"]))
    fu = [q.Field(L).load(c) for c in cu]
    fd = [q.Field(L).load(c) for c in cd]
    if nsm:  # sink smearing on the GPU: APE links, Gaussian steps on every time-slice
        gd, ga = q.Gauge(L, TH).load(u), q.Gauge(L, TH)
        q.ape3d(ga, gd, 0.5, nape)
        for f in fu + fd:
            for t in range(L[0]):
                q.gauss3d(f, ga, 4.0, t, nsm)
        ua = orc.ape3d(u, L, 0.5)
        for cols in (cu, cd):
            for k in range(12):
                for _ in range(nsm):
                    for t in range(L[0]):
                        cols[k] = orc.gauss3d(cols[k], ua, L, 4.0, t)
        gd.close()
        ga.close()
    corr = q.twop_proton(fu, fd, xsrc, t0, t1, TWOP_MOMS)
    want = orc.twop_proton(prop(cu), prop(cd), L, xsrc, t0, t1, TWOP_MOMS)
    assert np.max(np.abs(corr - want)) <= 1e-12 * np.max(np.abs(want))
    assert np.max(np.abs(corr - g["corr"])) <= 2e-6 * np.max(np.abs(g["corr"]))
    for f in fu + fd:
        f.close()


def test_solves_then_contraction_on_the_gpu(gpu, orc):
    L, xsrc = (8, 4, 4, 4), (2, 1, 3, 0)
    u = orc.gauge_synthetic(L, 61, EPS_PLAQ_060)
    g = q.Gauge(L, TH).load(u)
    b = q.Field(L)
    up, dn = [], []
    for mu_ in (0.02, -0.02):  # the two twisted-mass flavours
        cols = []
        for k in range(12):
            x = q.Field(L)
            b.point(xsrc, k // 3, k % 3)
            p = q.solve(x, b, g, 0.15, mu_, solver=q.SOLVER_CGNR_EO, inner_prec=q.F16, tol=1e-11)
            assert p.status == 0
            cols.append(x)
        (up if mu_ > 0 else dn).append(cols)
    up, dn = up[0], dn[0]
    corr = q.twop_proton(up, dn, xsrc, 0, L[0] - 1, [(0, 0, 0), (1, 0, 0)])
    V = int(np.prod(L))
    prop = lambda cs: np.stack([c.store() for c in cs]).reshape(4, 3, V, 4, 3, 2).transpose(2, 3, 0, 4, 1, 5)  # noqa
    want = orc.twop_proton(prop(up), prop(dn), L, xsrc, 0, L[0] - 1, [(0, 0, 0), (1, 0, 0)])
    assert np.max(np.abs(corr - want)) <= 1e-12 * np.max(np.abs(want))
    assert np.all(np.isfinite(corr)) and abs(corr[1, 0]) > 0
    for f in up + dn + [b, g]:
        f.close()


def test_twop_rejects_bad_arguments(gpu):
    L = (4, 4, 4, 4)
    fs = [q.Field(L) for _ in range(12)]
    with pytest.raises(q.QcdGpuError):
        q.twop_proton(fs, fs, (0, 0, 0, 9), 0, 1, [(0, 0, 0)])  # source outside the lattice
    with pytest.raises(q.QcdGpuError):
        q.twop_proton(fs, fs, (0, 0, 0, 0), 0, 4, [(0, 0, 0)])  # t1 beyond L_t
    for f in fs:
        f.close()
