"""Poisson request stream driven through the request server (qcdgpu_server).

A stream is a seeded list of arrivals: each request draws a resident gauge
field (one per lattice volume), kappa ~ U[kappa_lo, kappa_hi], an RHS count
in [1, max_rhs] (the spin-colour columns of point sources at seeded
positions) and a target residual. `run_stream` submits each request when its
arrival time has passed, runs scheduling rounds, releases completed requests
and reports throughput (RHS solved per second of wall time) and the p50 / p99
latency from submission to the last RHS retired.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import Gauge, Server, OP_D

SERVE_VOLUMES = ((16, 8, 8, 8), (32, 16, 16, 16), (48, 24, 24, 24), (64, 32, 32, 32))
EPS_PLAQ_060 = 0.43374  # exp(i eps H) scale of the synthetic ensemble with mean plaquette 0.60


@dataclass
class Arrival:
    t: float
    tag: int
    gauge: int
    nrhs: int
    kappa: float
    tol: float
    seed: int


def make_stream(rate_hz: float, duration_s: float, n_gauges: int, seed: int = 0, max_rhs: int = 48,
                kappa_range=(0.14, 0.155), tols=(1e-8, 1e-10), weights=None) -> list[Arrival]:
    """Seeded Poisson arrivals over [0, duration_s)."""
    rng = np.random.default_rng(seed)
    out, t, tag = [], 0.0, 0
    w = None if weights is None else np.asarray(weights, float) / np.sum(weights)
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            break
        out.append(Arrival(t=t, tag=tag, gauge=int(rng.choice(n_gauges, p=w)), nrhs=int(rng.integers(1, max_rhs + 1)),
                           kappa=float(rng.uniform(*kappa_range)), tol=float(rng.choice(tols)),
                           seed=int(rng.integers(1 << 62))))
        tag += 1
    return out


def build_gauges(volumes=SERVE_VOLUMES, theta=(np.pi, 0.0, 0.0, 0.0), eps=EPS_PLAQ_060):
    """One resident synthetic FP64 gauge field per volume (seeds 0, 1, ...)."""
    return [Gauge(L, theta).synthetic(i, eps) for i, L in enumerate(volumes)]


def run_stream(server: Server, gauge_ids: list[int], arrivals: list[Arrival], max_wall_s: float = 600.0,
               maxiter: int = 20000) -> dict:
    t0 = time.perf_counter()
    pending = list(arrivals)
    submitted = completed = rhs_done = rhs_iters = 0
    lat, queue, worst_res, statuses, iters = [], [], 0.0, {}, []
    while True:
        now = time.perf_counter() - t0
        while pending and pending[0].t <= now:
            a = pending.pop(0)
            server.submit(gauge_ids[a.gauge], a.nrhs, a.kappa, 0.0, OP_D, a.tol, tag=a.tag, seed=a.seed,
                          maxiter=maxiter)
            submitted += 1
        server.progress()
        for r in server.poll():
            completed += 1
            rhs_done += r["nrhs"]
            lat.append(r["latency_s"])
            queue.append(r["queue_s"])
            iters.append(r["max_iters"])
            rhs_iters += r["total_iters"]
            worst_res = max(worst_res, r["max_true_residual"])
            statuses[r["status"]] = statuses.get(r["status"], 0) + 1
            server.release(r["tag"])
        st = server.stats()
        if not pending and st["queued"] == 0 and st["active_rhs"] == 0 and completed == submitted:
            break
        if time.perf_counter() - t0 > max_wall_s:
            break
        if st["queued"] == 0 and st["active_rhs"] == 0 and pending:
            time.sleep(max(0.0, min(pending[0].t - (time.perf_counter() - t0), 0.01)))
    wall = time.perf_counter() - t0
    lat_a = np.array(lat) if lat else np.array([np.nan])
    return dict(requests=len(arrivals), completed=completed, rhs_solved=rhs_done, wall_s=wall,
                rhs_solves_per_s=rhs_done / wall if wall > 0 else 0.0,
                p50_s=float(np.percentile(lat_a, 50)), p99_s=float(np.percentile(lat_a, 99)),
                mean_queue_s=float(np.mean(queue)) if queue else None, worst_true_residual=worst_res,
                statuses=statuses, max_iters=int(max(iters)) if iters else 0, rhs_iterations=rhs_iters,
                mean_iters_per_rhs=rhs_iters / rhs_done if rhs_done else None,
                rhs_iterations_per_s=rhs_iters / wall if wall > 0 else 0.0)
