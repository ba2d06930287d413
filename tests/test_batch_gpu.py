"""Batched multi-RHS solver with continuous admission (qcdgpu_batch).

Every right-hand side is checked by its FP64 true residual computed by the
oracle, so the bar is the same as for the single-RHS solvers: |b - op x| / |b|
<= tol for each request, whatever it was batched with."""
import numpy as np
import pytest

import qcd_gb300 as q
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
L = (16, 8, 8, 8)
TH = (np.pi, 0.0, 0.0, 0.0)


def _run(batch, pending, max_steps=4000):
    """Feed (tag, x, b, kappa, mu, op, tol) requests as slots free up; returns {tag: (status, iters, res)}."""
    out = {}
    queue = list(pending)
    for _ in range(max_steps):
        while queue and batch.free_slots > 0:
            tag, fx, fb, kappa, mu, op, tol = queue.pop(0)
            k = batch.add(fx, fb, kappa, mu, op, tol=tol, maxiter=20000, tag=tag)
            assert k >= 0
        for tag, st, it, res in batch.poll():
            out[tag] = (st, it, res)
        if not queue and batch.active == 0:
            break
        batch.step(16)
    for tag, st, it, res in batch.poll():
        out[tag] = (st, it, res)
    return out


@pytest.fixture(params=[False, True], ids=["full", "eo"])
def eo(request):
    return request.param


def test_batch_mixed_kappa_mu_op_each_converges(gpu, orc, eo):
    u = orc.gauge_synthetic(L, 11, EPS_PLAQ_060)
    g = q.Gauge(L, TH).load(u)
    params = [(0.15, 0.0, q.OP_D, 1e-10), (0.14, 0.02, q.OP_D, 1e-10), (0.155, 0.0, q.OP_D, 1e-8),
              (0.145, 0.01, q.OP_Q, 1e-10), (0.15, 0.0, q.OP_Q, 1e-9), (0.12, 0.0, q.OP_D, 1e-10)]
    reqs, fields, srcs = [], [], []
    for i, (kappa, mu, op, tol) in enumerate(params):
        b = orc.gaussian_spinor(L, 300 + i)
        fb, fx = q.Field(L).load(b), q.Field(L)
        srcs.append(b)
        fields += [fb, fx]
        reqs.append((i, fx, fb, kappa, mu, op, tol))
    batch = q.Batch(g, 8, eo=eo)
    res = _run(batch, reqs)
    if not eo:
        assert q.mrhs_tuned(L, 8) is not None  # the operator variant was tuned before graph capture
    assert sorted(res) == list(range(len(params)))
    for i, (kappa, mu, op, tol) in enumerate(params):
        st, it, tr = res[i]
        assert st == 0, (i, res[i])
        x = reqs[i][1].store()
        true = orc.true_residual(x, srcs[i], u, L, TH, kappa, mu, op="Q" if op == q.OP_Q else "D")
        assert true <= tol, (i, true, tol)
        assert abs(true - tr) <= 1e-3 * tol + 1e-15
    batch.close()
    for f in fields + [g]:
        f.close()


def test_batch_continuous_admission_more_requests_than_slots(gpu, orc, eo):
    u = orc.gauge_synthetic(L, 12, EPS_PLAQ_060)
    g = q.Gauge(L, TH).load(u)
    n = 9
    reqs, fields, srcs = [], [], []
    for i in range(n):
        b = orc.gaussian_spinor(L, 400 + i) * (10.0 ** (i % 3 - 1))
        fb, fx = q.Field(L).load(b), q.Field(L)
        srcs.append(b)
        fields += [fb, fx]
        kappa = 0.13 + 0.0025 * i
        reqs.append((i, fx, fb, kappa, 0.0, q.OP_D, 1e-10))
    batch = q.Batch(g, 3, eo=eo)
    res = _run(batch, reqs)
    assert sorted(res) == list(range(n))
    for i in range(n):
        assert res[i][0] == 0, (i, res[i])
        x = reqs[i][1].store()
        assert orc.true_residual(x, srcs[i], u, L, TH, reqs[i][3]) <= 1e-10
    batch.close()
    for f in fields + [g]:
        f.close()


@pytest.mark.parametrize("source", ["gaussian", "point"])
def test_batch_result_independent_of_the_mix(gpu, orc, eo, source):
    """Per-slot reductions sum in a fixed order and the tensor-core product of
    one RHS row does not involve the others, so a request solved alone and in
    a mix (same capacity) gives bit-identical solutions. A point source spans
    many orders of magnitude over the sites, so its sums are not exact in any
    order: it would expose a summation order that depends on the mix."""
    u = orc.gauge_synthetic(L, 13, EPS_PLAQ_060)
    g = q.Gauge(L, TH).load(u)
    if source == "gaussian":
        b = orc.gaussian_spinor(L, 500)
    else:
        b = np.zeros((np.prod(L), 4, 3, 2))
        b[5, 1, 2, 0] = 1.0
    fb, fx_alone = q.Field(L).load(b), q.Field(L)
    batch = q.Batch(g, 4, eo=eo)
    _run(batch, [(0, fx_alone, fb, 0.15, 0.01, q.OP_D, 1e-10)])
    others = []
    reqs = []
    for i in range(3):
        ob = q.Field(L).load(orc.gaussian_spinor(L, 600 + i))
        ox = q.Field(L)
        others += [ob, ox]
        reqs.append((10 + i, ox, ob, 0.14 + 0.005 * i, 0.0, q.OP_D, 1e-10))
    fx_mix = q.Field(L)
    # the request under test enters the last slot, behind three others
    res = _run(batch, reqs + [(0, fx_mix, fb, 0.15, 0.01, q.OP_D, 1e-10)])
    assert res[0][0] == 0
    assert np.array_equal(fx_alone.store(), fx_mix.store())
    batch.close()
    for f in others + [fb, fx_alone, fx_mix, g]:
        f.close()


def test_batch_full_and_zero_rhs(gpu, orc):
    u = orc.gauge_synthetic(L, 14, EPS_PLAQ_060)
    g = q.Gauge(L, TH).load(u)
    batch = q.Batch(g, 1)
    fb = q.Field(L).load(orc.gaussian_spinor(L, 700))
    fz = q.Field(L)  # b = 0: solved by x = 0 without taking a slot
    x1, x2, xz = q.Field(L), q.Field(L), q.Field(L)
    assert batch.add(xz, fz, 0.15, tag=7) >= 0
    assert batch.active == 0
    assert batch.poll() == [(7, 0, 0, 0.0)]
    assert batch.add(x1, fb, 0.15, tag=1) == 0
    assert batch.add(x2, fb, 0.15, tag=2) == -1
    with pytest.raises(q.QcdGpuError):
        batch.add(x1, x1, 0.15)
    batch.close()
    for f in (fb, fz, x1, x2, xz, g):
        f.close()


def test_batch_eo_zero_rhs_and_fields_in_use(gpu, orc):
    """Even/odd batches keep a slot's c_e and A^{-1} b_o in its x until it
    retires: a zero right-hand side still returns x = 0 exactly, x may not
    be shared with a right-hand side in flight, and a converged x holds the
    solution over the work state."""
    u = orc.gauge_synthetic(L, 16, EPS_PLAQ_060)
    g = q.Gauge(L, TH).load(u)
    batch = q.Batch(g, 2, eo=True)
    b = orc.gaussian_spinor(L, 710)
    fb, fz = q.Field(L).load(b), q.Field(L)
    x1, x2, xz = q.Field(L), q.Field(L), q.Field(L)
    xz.load(orc.gaussian_spinor(L, 711))  # overwritten by the solve
    assert batch.add(xz, fz, 0.15, tag=7) >= 0
    assert batch.active == 0
    assert batch.poll() == [(7, 0, 0, 0.0)]
    assert not np.any(xz.store())
    assert batch.add(x1, fb, 0.15, tag=1) == 0
    with pytest.raises(q.QcdGpuError):
        batch.add(x1, fz, 0.15, tag=2)  # x of a right-hand side in flight
    with pytest.raises(q.QcdGpuError):
        batch.add(x2, x1, 0.15, tag=3)  # its x as a right-hand side
    with pytest.raises(q.QcdGpuError):
        batch.add(fb, fz, 0.15, tag=4)  # its right-hand side as x
    res = _run(batch, [])
    assert res[1][0] == 0
    tr = orc.true_residual(x1.store(), b, u, L, TH, 0.15)
    assert tr <= 1e-10, tr
    batch.close()
    for f in (fb, fz, x1, x2, xz, g):
        f.close()


def test_batch_eo_lattice_whose_x_cannot_hold_the_slot_fields(gpu, orc):
    """6x4x2x2: a full field pads to 128 sites and so does a half field, so x
    cannot hold c_e and A^{-1} b_o and the slot allocates them itself"""
    L2 = (6, 4, 2, 2)
    u = orc.gauge_synthetic(L2, 17, EPS_PLAQ_060)
    g = q.Gauge(L2, TH).load(u)
    batch = q.Batch(g, 2, eo=True)
    bs = [orc.gaussian_spinor(L2, 720 + i) for i in range(3)]
    fbs = [q.Field(L2).load(b) for b in bs]
    fxs = [q.Field(L2) for _ in bs]
    held = batch.nbytes()
    assert batch.add(fxs[0], fbs[0], 0.15, tag=0) == 0
    assert batch.nbytes() > held  # the slot's own c_e and A^{-1} b_o
    res = _run(batch, [(i, fxs[i], fbs[i], 0.14 + 0.005 * i, 0.01 * i, q.OP_D, 1e-10) for i in (1, 2)])
    assert sorted(res) == [0, 1, 2]
    for i in range(3):
        assert res[i][0] == 0, res[i]
        tr = orc.true_residual(fxs[i].store(), bs[i], u, L2, TH, 0.15 if i == 0 else 0.14 + 0.005 * i, 0.01 * i)
        assert tr <= 1e-10, (i, tr)
    assert batch.nbytes() == held
    batch.close()
    for f in fbs + fxs + [g]:
        f.close()


def test_even_odd_needs_every_extent_even(gpu, orc):
    """across the periodic boundary of an odd extent a site's neighbour has
    its own parity, so the checkerboard split does not hold: the even/odd
    batch and solve refuse such lattices, the full-lattice ones solve them"""
    L2 = (4, 3, 2, 2)
    u = orc.gauge_synthetic(L2, 18, EPS_PLAQ_060)
    g = q.Gauge(L2, TH).load(u)
    b = orc.gaussian_spinor(L2, 730)
    fb, fx = q.Field(L2).load(b), q.Field(L2)
    with pytest.raises(q.QcdGpuError):
        q.Batch(g, 2, eo=True)
    for solver in (q.SOLVER_CGNR_EO, q.SOLVER_BICGSTABL_EO):
        with pytest.raises(q.QcdGpuError):
            q.solve(fx, fb, g, 0.15, 0.0, solver=solver, inner_prec=q.F64, tol=1e-10)
    p = q.solve(fx, fb, g, 0.15, 0.0, solver=q.SOLVER_CGNR, inner_prec=q.F64, tol=1e-10)
    assert p.status == 0
    assert orc.true_residual(fx.store(), b, u, L2, TH, 0.15) <= 1e-10
    for f in (fb, fx, g):
        f.close()


def test_batch_on_tcgen05_kernel(gpu, orc, eo):
    """The batched solver on the tcgen05 multi-RHS kernel (16-slot capacity):
    every request converges to its FP64 true residual, and a request solved
    alone and behind three others gives bit-identical solutions."""
    import ctypes as C

    u = orc.gauge_synthetic(L, 15, EPS_PLAQ_060)
    g = q.Gauge(L, TH).load(u)
    q.set_mrhs_variant(2)
    try:
        params = [(0.15, 0.0, q.OP_D, 1e-10), (0.14, 0.02, q.OP_D, 1e-10), (0.155, 0.0, q.OP_Q, 1e-10),
                  (0.13, 0.0, q.OP_D, 1e-9), (0.145, 0.01, q.OP_D, 1e-10)]
        reqs, fields, srcs = [], [], []
        for i, (kappa, mu, op, tol) in enumerate(params):
            b = orc.gaussian_spinor(L, 700 + i) * (10.0 ** (i % 3 - 1))
            fb, fx = q.Field(L).load(b), q.Field(L)
            srcs.append(b)
            fields += [fb, fx]
            reqs.append((i, fx, fb, kappa, mu, op, tol))
        batch = q.Batch(g, 16, eo=eo)
        res = _run(batch, reqs)
        assert sorted(res) == list(range(len(params)))
        for i, (kappa, mu, op, tol) in enumerate(params):
            assert res[i][0] == 0, (i, res[i])
            x = reqs[i][1].store()
            true = orc.true_residual(x, srcs[i], u, L, TH, kappa, mu, op="Q" if op == q.OP_Q else "D")
            assert true <= tol, (i, true, tol)
        batch.close()
        # alone vs in a mix, same capacity
        b = np.zeros((np.prod(L), 4, 3, 2))
        b[7, 2, 1, 1] = 1.0
        fb, fx_alone, fx_mix = q.Field(L).load(b), q.Field(L), q.Field(L)
        fields += [fb, fx_alone, fx_mix]
        batch = q.Batch(g, 16, eo=eo)
        _run(batch, [(0, fx_alone, fb, 0.15, 0.01, q.OP_D, 1e-10)])
        mix = [(10 + i, reqs[i][1], reqs[i][2], 0.14, 0.0, q.OP_D, 1e-10) for i in range(3)]
        res = _run(batch, mix + [(0, fx_mix, fb, 0.15, 0.01, q.OP_D, 1e-10)])
        assert res[0][0] == 0
        assert np.array_equal(fx_alone.store(), fx_mix.store())
        batch.close()
        n = C.c_uint(0)
        assert q.lib().qcdgpu_mrhs_tc_timeouts(C.byref(n)) == 0 and n.value == 0
    finally:
        q.set_mrhs_variant(-1)
    for f in fields + [g]:
        f.close()
