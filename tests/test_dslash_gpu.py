"""GPU operator parity: the library's Wilson-TM operator against the
reference's own outputs (golden vectors) and the CPU oracle.

Tolerances: FP64 storage and arithmetic (native or float-float) <= 1e-13
relative per-site norm; FP32 storage <= 2e-6 and FP16(+norm) storage
<= 4e-3 relative global norm."""
import ctypes as C

import numpy as np
import pytest

import qcd_gb300 as q
from oracle.oracle import site_rel_err
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
TOL64 = 1e-13


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_op(L, theta, u, v, kappa, tm, op=q.OP_D, prec=q.F64, arith=q.ARITH_F64):
    g64 = q.Gauge(L, theta).load(u)
    g = g64 if prec == q.F64 else q.Gauge(L, theta, prec).convert_from(g64)
    src64 = q.Field(L).load(v)
    src = src64 if prec == q.F64 else q.Field(L, prec).copy_from(src64)
    out = q.Field(L, prec)
    q.dslash(out, src, g, kappa, tm, op, arith)
    out64 = out if prec == q.F64 else q.Field(L).copy_from(out)
    res = out64.store()
    recon = g64.recon
    for f in {id(x): x for x in (g64, g, src64, src, out, out64)}.values():
        f.close()
    return res, recon


@pytest.mark.parametrize("case", ["wilson_L6442", "wilson_L4444_theta"])
@pytest.mark.parametrize("arith", [q.ARITH_F64, q.ARITH_DF64], ids=["f64", "df64"])
def test_fp64_operator_matches_reference_golden(gpu, golden, case, arith):
    g = golden[case]
    L, th, kappa, tm = g["L"], g["theta"], float(g["kappa"]), float(g["tm"])
    out, recon = run_op(L, th, g["u"], g["v"], kappa, tm, q.OP_D, arith=arith)
    assert recon == 12  # synthetic links are SU(3): 12-real storage
    assert site_rel_err(out, g["out_TMOp"]) <= TOL64
    outq, _ = run_op(L, th, g["u"], g["v"], kappa, tm, q.OP_Q, arith=arith)
    assert site_rel_err(outq, g["out_Q"]) <= TOL64


@pytest.mark.parametrize("L", [(16, 8, 8, 8), (6, 4, 4, 2), (2, 2, 2, 2), (8, 6, 4, 10)])
def test_fp64_operator_vs_oracle(gpu, orc, L):
    th = (np.pi, 0.0, 0.2, 0.0)
    u = orc.gauge_synthetic(L, 21, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 22)
    for tm in (0.0, 0.07):
        ref = orc.dslash(v, u, L, th, kappa=0.15, tm=tm)
        out, _ = run_op(L, th, u, v, 0.15, tm)
        assert site_rel_err(out, ref) <= TOL64


@pytest.mark.parametrize("arith", [q.ARITH_F64, q.ARITH_DF64], ids=["f64", "df64"])
def test_pipelined_host_apply_matches_oracle(gpu, orc, arith):
    """qcd_applyWilsonTMOp / qcd_applyQTMOp on page-locked host vectors take
    the slab pipeline (copy in, operator, copy out per z-slab); with
    float-float arithmetic the operator reads and writes the host layout in
    place. Every slab count, including the periodic first/last slab pair,
    gives the oracle's result."""
    L = (6, 4, 4, 12)
    th = (np.pi, 0.0, 0.3, 0.0)
    kappa, tm = 0.15, 0.05
    m = 1.0 / (2.0 * kappa) - 4.0
    u_h = orc.gauge_synthetic(L, 31, EPS_PLAQ_060)
    v_h = orc.gaussian_spinor(L, 32)
    ref_d = orc.dslash(v_h, u_h, L, th, kappa=kappa, tm=tm)
    ref_q = orc.dslash(v_h, u_h, L, th, kappa=kappa, tm=tm, op="Q")
    geo = q.Geometry(L, th)
    v, Dv, u = q.Vector(geo), q.Vector(geo), q.GaugeField(geo)
    u.a[:] = u_h
    v.a[:] = v_h
    lib = q.lib()
    lib.qcdgpu_set_pipeline_slabs.argtypes = [C.c_int]
    assert lib.qcdgpu_set_f64_arith(arith) == 0
    try:
        for S in (3, 4, 6, 12, 0):
            assert lib.qcdgpu_set_pipeline_slabs(S) == 0
            Dv.a[:] = 0.0
            assert lib.qcd_applyWilsonTMOp(Dv.ref, v.ref, u.ref, m, tm) == 0
            assert site_rel_err(Dv.a, ref_d) <= TOL64, S
            Dv.a[:] = 0.0
            assert lib.qcd_applyQTMOp(Dv.ref, v.ref, u.ref, m, tm) == 0
            assert site_rel_err(Dv.a, ref_q) <= TOL64, S
    finally:
        lib.qcdgpu_set_pipeline_slabs(0)
        lib.qcdgpu_set_f64_arith(q.ARITH_DF64)  # the library default
        for o in (v, Dv, u):
            o.close()
        geo.close()


def test_fp64_operator_general_links_use_18_reals(gpu, orc):
    L = (4, 4, 2, 6)
    rng = np.random.default_rng(3)
    u = rng.normal(size=(np.prod(L), 4, 3, 3, 2))
    v = rng.normal(size=(np.prod(L), 4, 3, 2))
    th = (np.pi, 0, 0, 0)
    out, recon = run_op(L, th, u, v, 0.13, 0.2)
    assert recon == 18
    assert site_rel_err(out, orc.dslash(v, u, L, th, kappa=0.13, tm=0.2)) <= TOL64


def test_adjoint_and_normal_operator(gpu, orc):
    L = (8, 4, 4, 4)
    th = (np.pi, 0, 0, 0)
    u = orc.gauge_synthetic(L, 5, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 6)
    out, _ = run_op(L, th, u, v, 0.15, 0.1, q.OP_DDAG)
    assert site_rel_err(out, orc.dslash(v, u, L, th, kappa=0.15, tm=0.1, op="Ddag")) <= TOL64
    out, _ = run_op(L, th, u, v, 0.15, 0.1, q.OP_DDAGD)
    dd = orc.dslash(orc.dslash(v, u, L, th, kappa=0.15, tm=0.1), u, L, th, kappa=0.15, tm=0.1, op="Ddag")
    assert site_rel_err(out, dd) <= TOL64


@pytest.mark.parametrize("prec,tol", [(q.F32, 2e-6), (q.F16, 4e-3)])
def test_low_precision_operator(gpu, orc, prec, tol):
    L = (8, 8, 8, 8)
    th = (np.pi, 0, 0, 0)
    u = orc.gauge_synthetic(L, 7, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 8)
    ref = orc.dslash(v, u, L, th, kappa=0.15, tm=0.05)
    for op, o in ((q.OP_D, "D"), (q.OP_DDAG, "Ddag")):
        ref = orc.dslash(v, u, L, th, kappa=0.15, tm=0.05, op=o)
        out, _ = run_op(L, th, u, v, 0.15, 0.05, op, prec=prec)
        assert rel(out, ref) <= tol
    dd = orc.dslash(orc.dslash(v, u, L, th, kappa=0.15, tm=0.05), u, L, th, kappa=0.15, tm=0.05, op="Ddag")
    out, _ = run_op(L, th, u, v, 0.15, 0.05, q.OP_DDAGD, prec=prec)
    assert rel(out, dd) <= 2 * tol


def test_dropin_operator_entry_points(gpu, golden):
    """qcd_applyWilsonTMOp & co. on host structs reproduce the reference."""
    g = golden["wilson_L6442"]
    L, th, kappa, tm = g["L"], g["theta"], float(g["kappa"]), float(g["tm"])
    m = 1.0 / (2.0 * kappa) - 4.0
    geo = q.Geometry(L, th)
    v, Dv = q.Vector(geo), q.Vector(geo)
    u = q.GaugeField(geo)
    u.a[:] = g["u"]
    v.a[:] = g["v"]
    lib = q.lib()
    for name, key in (("qcd_applyWilsonTMOp", "out_TMOp"), ("qcd_applyWilsonTMOpNoOptim", "out_NoOptim"),
                      ("qcd_applyWilsonTMOpNoScripts", "out_NoScripts"), ("qcd_applyQTMOp", "out_Q")):
        Dv.a[:] = 0
        assert getattr(lib, name)(Dv.ref, v.ref, u.ref, m, tm) == 0
        assert site_rel_err(Dv.a, g[key]) <= TOL64
    # host data changed behind the library's back is picked up (no stale mirror)
    v.a[:] = 2.0 * g["v"]
    assert lib.qcd_applyWilsonTMOp(Dv.ref, v.ref, u.ref, m, tm) == 0
    assert site_rel_err(Dv.a, 2.0 * g["out_TMOp"]) <= TOL64
    # residency: resident gauge + resident input, explicit copies
    assert lib.qcdgpu_gauge_upload(u.ref) == 0
    assert lib.qcdgpu_vector_make_resident(v.ref) == 0
    v.a[:] = 0.0  # host copy is now stale by design
    assert lib.qcd_applyWilsonTMOp(Dv.ref, v.ref, u.ref, m, tm) == 0
    assert site_rel_err(Dv.a, 2.0 * g["out_TMOp"]) <= TOL64
    assert lib.qcdgpu_vector_to_host(v.ref) == 0
    assert np.array_equal(v.a, 2.0 * g["v"])
    assert lib.qcdgpu_vector_release(v.ref) == 0
    assert lib.qcdgpu_gauge_release(u.ref) == 0
    for o in (v, Dv, u):
        o.close()
    geo.close()


def test_generators_match_oracle(gpu, orc):
    L = (8, 4, 4, 6)
    g = q.Gauge(L).synthetic(31, EPS_PLAQ_060)
    u = g.store()
    ref = orc.gauge_synthetic(L, 31, EPS_PLAQ_060)
    assert np.max(np.abs(u - ref)) <= 1e-13
    assert g.recon == 12
    assert abs(g.plaquette() - orc.plaquette(ref, L)) <= 1e-13
    f = q.Field(L).gaussian(32)
    assert np.max(np.abs(f.store() - orc.gaussian_spinor(L, 32))) <= 1e-12
    f.point((1, 2, 3, 4), 2, 1)
    p = f.store()
    assert p[1 + 8 * (2 + 4 * (3 + 4 * 4)), 2, 1, 0] == 1.0 and np.sum(np.abs(p)) == 1.0
    g.close()
    f.close()


def test_operator_rejects_bad_arguments(gpu):
    L = (4, 4, 4, 4)
    a, b = q.Field(L), q.Field((4, 4, 4, 8))
    g = q.Gauge(L).synthetic(1, 0.4)
    with pytest.raises(q.QcdGpuError):
        q.dslash(a, a, g, 0.15)  # aliasing
    with pytest.raises(q.QcdGpuError):
        q.dslash(a, b, g, 0.15)  # shapes
    c = q.Field(L, q.F32)
    with pytest.raises(q.QcdGpuError):
        q.dslash(c, a, g, 0.15)  # precisions
    for f in (a, b, c, g):
        f.close()
