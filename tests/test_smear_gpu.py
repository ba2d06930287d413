"""Source construction on the GPU against the oracle (which is pinned to the
reference's qcd_apeSmear3d / qcd_gaussIteration3d / qcd_calculatePlaquette):
APE links and Gaussian-smeared spinors to 1e-12 relative (the projection's
Newton iteration stops at a relative step of 1e-15), the plaquette to 1e-14."""
import numpy as np
import pytest

import qcd_gb300 as q
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
L = (8, 4, 6, 4)
TH = (np.pi, 0.0, 0.0, 0.0)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("steps", [1, 4])
def test_ape3d_matches_oracle(gpu, orc, steps):
    u = orc.gauge_synthetic(L, 31, EPS_PLAQ_060)
    ref = u
    for _ in range(steps):
        ref = orc.ape3d(ref, L, 0.5)
    g, o = q.Gauge(L, TH).load(u), q.Gauge(L, TH)
    q.ape3d(o, g, 0.5, steps)
    assert rel(o.store(), ref) <= 1e-12 * steps
    assert abs(o.plaquette() - orc.plaquette(ref, L)) <= 1e-13
    g.close()
    o.close()


def test_gauss3d_matches_oracle(gpu, orc):
    u = orc.gauge_synthetic(L, 32, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 33)
    ref = v
    for _ in range(3):
        ref = orc.gauss3d(ref, u, L, 4.0, 5)
    g, f = q.Gauge(L, TH).load(u), q.Field(L).load(v)
    q.gauss3d(f, g, 4.0, 5, 3)
    out = f.store()
    assert rel(out, ref) <= 1e-13
    # other time-slices are untouched
    t = np.arange(out.shape[0]) % L[0]
    assert np.array_equal(out[t != 5], v[t != 5])
    g.close()
    f.close()


def test_smeared_source_matches_oracle(gpu, orc):
    u = orc.gauge_synthetic(L, 34, EPS_PLAQ_060)
    ua = u
    for _ in range(2):
        ua = orc.ape3d(ua, L, 0.5)
    x = (3, 1, 2, 0)
    src = np.zeros((np.prod(L), 4, 3, 2))
    site = x[0] + L[0] * (x[1] + L[1] * (x[2] + L[2] * x[3]))
    src[site, 2, 1, 0] = 1.0
    for _ in range(5):
        src = orc.gauss3d(src, ua, L, 4.0, x[0])
    g, f = q.Gauge(L, TH).load(u), q.Field(L)
    q.smeared_source(f, g, x, 2, 1, 0.5, 2, 4.0, 5)
    assert rel(f.store(), src) <= 1e-12
    g.close()
    f.close()


def test_dropin_smearing_and_plaquette(gpu, orc):
    u = orc.gauge_synthetic(L, 35, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 36)
    geo = q.Geometry(L, TH)
    gu, ga, vec = q.GaugeField(geo), q.GaugeField(geo), q.Vector(geo)
    gu.a[:] = u.reshape(gu.a.shape)
    vec.a[:] = v.reshape(vec.a.shape)
    assert q.lib().qcd_apeSmear3d(ga.ref, gu.ref, 0.5) == 0
    assert rel(np.array(ga.a).reshape(u.shape), orc.ape3d(u, L, 0.5)) <= 1e-12
    assert q.lib().qcd_apeSmear3d(gu.ref, gu.ref, 0.5) == 1  # in place is rejected
    assert q.lib().qcd_gaussIteration3d(vec.ref, gu.ref, 4.0, 2) == 0
    assert rel(np.array(vec.a).reshape(v.shape), orc.gauss3d(v, u, L, 4.0, 2)) <= 1e-13
    assert abs(q.lib().qcd_calculatePlaquette(gu.ref) - orc.plaquette(u, L)) <= 1e-14
    for o in (gu, ga, vec):
        o.close()
    geo.close()
