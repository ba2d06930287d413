"""GPU BLAS-1 parity through the drop-in entry points (qcd_blas.c:137-492)
against the reference's golden outputs and the oracle."""
import numpy as np
import pytest

import qcd_gb300 as q

pytestmark = pytest.mark.gpu


def test_dropin_blas(gpu, orc, golden):
    g = golden["wilson_L4444_theta"]
    geo = q.Geometry(g["L"], g["theta"])
    lib = q.lib()
    v, w, o = q.Vector(geo), q.Vector(geo), q.Vector(geo)
    v.a[:] = g["v"]
    w.a[:] = g["w"]
    # norm and dot: FP64 accumulation in a different order -> 1e-14 relative
    assert abs(lib.qcd_normVector(v.ref) - float(g["norm_v"])) <= 1e-14 * float(g["norm_v"])
    d = lib.qcd_mulAdjointVectorVector(v.ref, w.ref)
    dr = complex(*g["dot_vw"])
    assert abs(complex(d.re, d.im) - dr) <= 1e-13 * np.linalg.norm(g["v"]) * np.linalg.norm(g["w"])
    a = complex(*g["axpy_a"])
    lib.qcd_axpyVector(o.ref, q.QcdComplex16(a.real, a.imag), v.ref, w.ref)
    assert np.max(np.abs(o.a - g["axpy_vw"])) <= 1e-15 * np.max(np.abs(g["axpy_vw"]))
    # in-place forms as invert.c uses them: y = a x + y
    o.a[:] = g["w"]
    lib.qcd_axpyVector(o.ref, q.QcdComplex16(a.real, a.imag), v.ref, o.ref)
    assert np.max(np.abs(o.a - g["axpy_vw"])) <= 1e-15 * np.max(np.abs(g["axpy_vw"]))
    lib.qcd_addVector(o.ref, v.ref, w.ref)
    assert np.array_equal(o.a, g["v"] + g["w"])
    lib.qcd_subVector(o.ref, v.ref, w.ref)
    assert np.array_equal(o.a, g["v"] - g["w"])
    lib.qcd_copyVector(o.ref, v.ref)
    assert np.array_equal(o.a, g["v"])
    lib.qcd_scaleVector(o.ref, 0.25)
    assert np.array_equal(o.a, 0.25 * g["v"])
    o.a[:] = g["v"]
    c = 0.5 + 2j
    lib.qcd_mulVectorC(o.ref, q.QcdComplex16(c.real, c.imag))
    ref = (g["v"][..., 0] + 1j * g["v"][..., 1]) * c
    assert np.max(np.abs(o.a[..., 0] + 1j * o.a[..., 1] - ref)) <= 1e-15 * np.max(np.abs(ref))
    lib.qcd_zeroVector(o.ref)
    assert not o.a.any()
    lib.qcd_setVector(o.ref, q.QcdComplex16(1.5, -2.0))
    assert np.all(o.a[..., 0] == 1.5) and np.all(o.a[..., 1] == -2.0)
    o.a[:] = g["v"]
    lib.qcd_gamma5Vector(o.ref)
    assert np.array_equal(o.a[:, :2], g["v"][:, :2]) and np.array_equal(o.a[:, 2:], -g["v"][:, 2:])
    for x in (v, w, o):
        x.close()
    geo.close()


@pytest.mark.parametrize("prec,tol", [(q.F64, 1e-14), (q.F32, 1e-6), (q.F16, 2e-3)])
def test_device_reductions(gpu, orc, prec, tol):
    L = (16, 8, 8, 8)
    a = orc.gaussian_spinor(L, 1)
    b = orc.gaussian_spinor(L, 2)
    fa64, fb64 = q.Field(L).load(a), q.Field(L).load(b)
    fa = fa64 if prec == q.F64 else q.Field(L, prec).copy_from(fa64)
    fb = fb64 if prec == q.F64 else q.Field(L, prec).copy_from(fb64)
    n2 = fa.norm2()
    # reference: correctly rounded sum of squares (the oracle's sequential sum
    # over 3M terms carries ~1e-14 relative rounding of its own)
    import math

    exact = math.fsum((a.ravel() ** 2).tolist())
    assert abs(n2 - exact) <= tol * exact
    d = fa.dot(fb)
    ref = orc.dot(a, b)
    assert abs(d - ref) <= tol * orc.norm(a) * orc.norm(b)
    # reductions are deterministic run to run
    assert fa.norm2() == n2 and fa.dot(fb) == d
    for f in {id(x): x for x in (fa64, fb64, fa, fb)}.values():
        f.close()
