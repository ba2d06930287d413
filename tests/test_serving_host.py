"""Host side of the serving stream: seeded Poisson arrivals (no GPU)."""
import numpy as np

from qcd_gb300.serving import make_stream


def test_stream_is_seeded_and_in_range():
    a = make_stream(5.0, 60.0, 4, seed=3)
    b = make_stream(5.0, 60.0, 4, seed=3)
    assert [(x.t, x.gauge, x.nrhs, x.kappa, x.tol, x.seed) for x in a] == \
        [(x.t, x.gauge, x.nrhs, x.kappa, x.tol, x.seed) for x in b]
    assert all(0.0 < x.t < 60.0 for x in a)
    assert all(0.14 <= x.kappa <= 0.155 for x in a)
    assert all(1 <= x.nrhs <= 48 for x in a)
    assert {x.tol for x in a} == {1e-8, 1e-10}
    assert {x.gauge for x in a} == {0, 1, 2, 3}
    assert [x.tag for x in a] == list(range(len(a)))
    assert np.all(np.diff([x.t for x in a]) > 0)


def test_stream_rate_matches_poisson_mean():
    a = make_stream(20.0, 500.0, 4, seed=1)
    # 10000 expected arrivals: the count is within 4 sigma (sigma = 100)
    assert abs(len(a) - 10000) < 400
    gaps = np.diff([x.t for x in a])
    assert abs(np.mean(gaps) - 0.05) < 0.002


def test_stream_weights_select_gauges():
    a = make_stream(10.0, 100.0, 4, seed=2, weights=(1, 0, 0, 1))
    assert {x.gauge for x in a} == {0, 3}
