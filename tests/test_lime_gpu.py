"""LIME / ILDG / ETMC file I/O through the drop-in entry points and the
device API. Files are built independently in Python from the format and
qcd_lib's data order (tests/lime_util.py); reads must reproduce the arrays
exactly (FP64) or to FP32 rounding, and files the library writes must parse
back to the same records and bytes."""
import ctypes as C

import numpy as np
import pytest

import qcd_gb300 as q
from tests import lime_util
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
L = (8, 4, 6, 2)
TH = (np.pi, 0.0, 0.0, 0.0)


def _lib():
    lib = q.lib()
    up, vp = C.POINTER(q.QcdGaugeField), C.POINTER(q.QcdVector)
    lib.qcd_getGaugeLime.argtypes = [C.c_char_p, up]
    lib.qcd_writeGaugeLime.argtypes = [C.c_char_p, up, C.c_char_p]
    lib.qcd_getGaugeField.argtypes = [C.c_char_p, C.c_int, up]
    lib.qcd_getVectorLime.argtypes = [C.c_char_p, vp]
    lib.qcd_writeVectorLime.argtypes = [C.c_char_p, C.c_int, vp]
    for n in ("qcdgpu_gauge_load_lime", "qcdgpu_field_load_lime"):
        getattr(lib, n).argtypes = [C.c_void_p, C.c_char_p]
    lib.qcdgpu_gauge_save_lime.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
    lib.qcdgpu_field_save_lime.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    return lib


@pytest.mark.parametrize("prec", [64, 32])
def test_read_ildg_gauge_written_from_the_format(gpu, orc, tmp_path, prec):
    u = orc.gauge_synthetic(L, 51, EPS_PLAQ_060)
    path = tmp_path / "conf.lime"
    path.write_bytes(lime_util.ildg_file(u, L, prec))
    lib = _lib()
    geo = q.Geometry(L, TH)
    gf = q.GaugeField(geo)
    assert lib.qcd_getGaugeField(str(path).encode(), 0, gf.ref) == 0
    got = np.array(gf.a).reshape(u.shape)
    want = u if prec == 64 else u.astype(np.float32).astype(np.float64)
    assert np.array_equal(got, want)
    assert lib.qcd_getGaugeField(str(path).encode(), 1, gf.ref) == 1  # unknown type
    # device API: the same file straight into a device field
    g = q.Gauge(L, TH)
    assert lib.qcdgpu_gauge_load_lime(g.h, str(path).encode()) == 0
    assert np.array_equal(g.store(), want)
    if prec == 64:
        assert abs(g.plaquette() - orc.plaquette(u, L)) <= 1e-14
    gf.close()
    geo.close()
    g.close()


def test_gauge_write_then_read_round_trip(gpu, orc, tmp_path):
    u = orc.gauge_synthetic(L, 52, EPS_PLAQ_060)
    lib = _lib()
    geo = q.Geometry(L, TH)
    a, b = q.GaugeField(geo), q.GaugeField(geo)
    a.a[:] = u.reshape(a.a.shape)
    path = tmp_path / "w.lime"
    assert lib.qcd_writeGaugeLime(str(path).encode(), a.ref, b"written by the test") == 0
    recs = lime_util.parse(path.read_bytes())
    assert [(r[0], r[1], r[2]) for r in recs] == [("ildg-format", True, False), ("xlf-info", False, False),
                                                  ("ildg-binary-data", False, True)]
    assert b"<precision> 64 </precision>" in recs[0][3] and recs[1][3] == b"written by the test"
    assert recs[2][3] == lime_util.ildg_payload(u, L, 64)
    assert lib.qcd_getGaugeLime(str(path).encode(), b.ref) == 0
    assert np.array_equal(np.array(b.a), np.array(a.a))
    a.close()
    b.close()
    geo.close()


@pytest.mark.parametrize("prec", [64, 32])
def test_etmc_spinor_read_and_write(gpu, orc, tmp_path, prec):
    v = orc.gaussian_spinor(L, 53)
    path = tmp_path / "prop.lime"
    path.write_bytes(lime_util.etmc_file(v, L, prec))
    lib = _lib()
    geo = q.Geometry(L, TH)
    vec = q.Vector(geo)
    assert lib.qcd_getVectorLime(str(path).encode(), vec.ref) == 0
    want = v if prec == 64 else v.astype(np.float32).astype(np.float64)
    assert np.array_equal(np.array(vec.a).reshape(v.shape), want)
    out = tmp_path / "out.lime"
    assert lib.qcd_writeVectorLime(str(out).encode(), 4, vec.ref) == 0  # qcd_SOURCE_LIME
    recs = lime_util.parse(out.read_bytes())
    assert [r[0] for r in recs] == ["source-type", "etmc-source-format", "scidac-binary-data"]
    assert recs[2][3] == lime_util.etmc_payload(want, L, 64)
    f = q.Field(L)
    assert lib.qcdgpu_field_load_lime(f.h, str(out).encode()) == 0
    assert np.array_equal(f.store(), want)
    vec.close()
    geo.close()
    f.close()


def test_lattice_mismatch_is_an_error(gpu, orc, tmp_path):
    u = orc.gauge_synthetic(L, 54, EPS_PLAQ_060)
    path = tmp_path / "conf.lime"
    path.write_bytes(lime_util.ildg_file(u, L))
    g = q.Gauge((8, 4, 6, 4), TH)
    assert _lib().qcdgpu_gauge_load_lime(g.h, str(path).encode()) == 1
    assert _lib().qcdgpu_gauge_load_lime(g.h, str(tmp_path / "missing.lime").encode()) == 1
    g.close()
