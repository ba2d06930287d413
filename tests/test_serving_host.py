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


class _FakeServer:
    """Stands in for qcdgpu_server on the host: each progress call retires
    the oldest request; a request of n RHS reports 10 * (c + 1) iterations
    for its column c (max 10 n, total 5 n (n + 1))."""

    def __init__(self):
        self.waiting, self.done, self.released = [], [], []

    def submit(self, gid, nrhs, kappa, mu, op, tol, tag=0, seed=0, maxiter=0):
        self.waiting.append((tag, nrhs, tol))

    def progress(self):
        if self.waiting:
            tag, n, tol = self.waiting.pop(0)
            self.done.append(dict(tag=tag, status=0, nrhs=n, max_iters=10 * n, max_true_residual=0.5 * tol,
                                  queue_s=0.0, latency_s=0.001 * n, total_iters=5 * n * (n + 1)))

    def poll(self):
        out, self.done = self.done, []
        return out

    def release(self, tag):
        self.released.append(tag)

    def stats(self):
        return dict(bytes_used=0, queued=0, active_rhs=sum(w[1] for w in self.waiting))


def test_run_stream_accounts_every_request_and_iteration():
    from qcd_gb300.serving import run_stream

    arr = make_stream(200.0, 0.1, 2, seed=5)
    srv = _FakeServer()
    res = run_stream(srv, [0, 1], arr, max_wall_s=30.0)
    n = [a.nrhs for a in arr]
    assert res["requests"] == res["completed"] == len(arr)
    assert sorted(srv.released) == [a.tag for a in arr]
    assert res["rhs_solved"] == sum(n)
    assert res["rhs_iterations"] == sum(5 * k * (k + 1) for k in n)
    assert res["mean_iters_per_rhs"] == res["rhs_iterations"] / sum(n)
    assert res["max_iters"] == 10 * max(n)
    assert res["statuses"] == {0: len(arr)}
    assert res["worst_true_residual"] == max(0.5 * a.tol for a in arr)
    assert res["rhs_iterations_per_s"] == res["rhs_iterations"] / res["wall_s"]
