"""Stochastic sources (qcd_stochastic.c:8-58): Z4 and Z2 noise on the GPU.

The reference draws its noise from GSL's ranlux, which is not available, so
parity of the streams themselves is not pinned; the library's counter-based
stream is pinned to the oracle's restatement of it bit for bit, and the
distribution is checked: every component exactly one of the allowed values,
each value about equally often, zeros off the chosen time-slice, and
independent draws on successive qcd_z2Vector calls."""
import numpy as np
import pytest

import qcd_gb300 as q

pytestmark = pytest.mark.gpu
L = (8, 6, 4, 4)


@pytest.mark.parametrize("kind", [4, 2])
@pytest.mark.parametrize("t_slice", [-1, 3])
def test_noise_matches_oracle_stream(gpu, orc, kind, t_slice):
    f = q.Field(L).noise(77, t_slice, kind)
    got = f.store()
    want = orc.noise_spinor(L, 77, t_slice, kind)
    assert np.array_equal(got, want)
    f.close()


def test_noise_distribution(gpu):
    Lb = (16, 16, 16, 16)
    f = q.Field(Lb).noise(5, -1, 4)
    z = f.store().reshape(-1, 2)
    c = z[:, 0] + 1j * z[:, 1]
    vals = np.array([1, 1j, -1, -1j])
    counts = np.array([np.sum(c == v) for v in vals])
    assert counts.sum() == c.size  # nothing outside Z4
    n = c.size / 4
    assert np.all(np.abs(counts - n) <= 5 * np.sqrt(n * 0.75))
    f.noise(6, -1, 2)
    z2 = f.store()
    assert np.all(z2[..., 1] == 0) and np.all(np.abs(z2[..., 0]) == 1)
    assert abs(np.mean(z2[..., 0])) <= 5 / np.sqrt(z2[..., 0].size)
    f.close()


def test_dropin_z2vector_time_dilution_and_fresh_draws(gpu):
    lib = q.lib()
    geo = q.Geometry(L)
    v = q.Vector(geo)
    try:
        assert lib.qcdgpu_set_noise_seed(11) == 0
        lib.qcd_z2Vector(v.ref, 2)
        a = v.a.copy()
        t = np.arange(np.prod(L)) % L[0]
        assert np.all(a[t != 2] == 0)
        on = a[t == 2]
        c = on[..., 0] + 1j * on[..., 1]
        assert np.all(np.isin(c, [1, 1j, -1, -1j]))
        lib.qcd_z2Vector(v.ref, 2)
        assert not np.array_equal(v.a, a)  # a new draw every call
        assert lib.qcdgpu_set_noise_seed(11) == 0
        lib.qcd_z2Vector(v.ref, 2)
        assert np.array_equal(v.a, a)  # the seed restarts the stream
        lib.qcd_z2Vector(v.ref, -1)
        assert np.all(np.abs(v.a[..., 0]) + np.abs(v.a[..., 1]) == 1)
        lib.qcd_z2Vector(v.ref, L[0])  # past the lattice: a zero vector, as the reference leaves it
        assert np.all(v.a == 0)
    finally:
        v.close()
        geo.close()
