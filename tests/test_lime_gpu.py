"""LIME / ILDG / ETMC and legacy CMI / HMC / HMCV file I/O through the drop-in
entry points and the device API. Inputs are files the reference's own
qcd_io.c wrote (tests/golden/io_L4235.npz) and files built in Python from the
format models (tests/lime_util.py, tests/legacy_formats.py, which the host
tests pin to the reference's readers); reads must reproduce the arrays
exactly (FP64) or to FP32 rounding, and files the library writes must match
the reference's bytes."""
import ctypes as C
import struct

import numpy as np
import pytest

import qcd_gb300 as q
from tests import legacy_formats, lime_util
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


def _vlib():
    lib = _lib()
    vp = C.POINTER(q.QcdVector)
    for n in ("qcd_getVectorCMI", "qcd_getVectorHMC", "qcd_getVectorHMCV", "qcd_writeVectorCMI"):
        getattr(lib, n).argtypes = [C.c_char_p, C.c_uint16, C.c_uint16, vp]
    for n in ("qcd_getVector", "qcd_writeVector"):
        getattr(lib, n).argtypes = [C.c_char_p, C.c_int, C.c_uint16, C.c_uint16, vp]
    return lib


def test_reference_written_files_read_and_written_bit_exactly(gpu, golden, tmp_path):
    """files written by the reference's own qcd_io.c (tests/golden/io_L4235.npz):
    the library reads them to the arrays they were written from, and writes
    the same arrays to the same bytes"""
    g = golden["io_L4235"]
    Lg = tuple(int(x) for x in g["L"])
    lib = _vlib()
    geo = q.Geometry(Lg, TH)
    gf, vec = q.GaugeField(geo), q.Vector(geo)
    files = {}
    for key in ("conf_lime", "prop_lime", "source_lime", "vec_cmi"):
        files[key] = tmp_path / key
        files[key].write_bytes(g[key].tobytes())
    assert lib.qcd_getGaugeField(str(files["conf_lime"]).encode(), 0, gf.ref) == 0
    assert np.array_equal(np.array(gf.a).reshape(g["u"].shape), g["u"])
    for key in ("prop_lime", "source_lime"):
        vec.a[:] = 0
        assert lib.qcd_getVector(str(files[key]).encode(), 3, 0, 0, vec.ref) == 0
        assert np.array_equal(np.array(vec.a).reshape(g["v"].shape), g["v"]), key
    v32 = g["v"].astype(np.float32).astype(np.float64)
    for nu, c in ((0, 0), (2, 1)):
        vec.a[:] = 0
        assert lib.qcd_getVectorCMI(str(files["vec_cmi"]).encode(), nu, c, vec.ref) == 0
        assert np.array_equal(np.array(vec.a).reshape(v32.shape), v32)
    vec.a[:] = 0
    assert lib.qcd_getVector(str(files["vec_cmi"]).encode(), 0, 0, 0, vec.ref) == 0
    assert np.array_equal(np.array(vec.a).reshape(v32.shape), v32)
    # writers: the same arrays to the same bytes
    out = tmp_path / "out"
    assert lib.qcd_writeGaugeLime(str(out).encode(), gf.ref, g["message"].tobytes()) == 0
    assert out.read_bytes() == files["conf_lime"].read_bytes()
    vec.a[:] = g["v"].reshape(vec.a.shape)
    for t, key in ((3, "prop_lime"), (4, "source_lime"), (0, "vec_cmi")):
        assert lib.qcd_writeVector(str(out).encode(), t, 0, 0, vec.ref) == 0
        assert out.read_bytes() == files[key].read_bytes(), key
    assert lib.qcd_writeVectorCMI(str(out).encode(), 1, 2, vec.ref) == 0
    assert out.read_bytes() == files["vec_cmi"].read_bytes()
    assert lib.qcd_writeVector(str(out).encode(), 1, 0, 0, vec.ref) == 1  # no HMC writer
    gf.close()
    vec.close()
    geo.close()


def test_legacy_hmc_and_hmcv_vectors(gpu, orc, tmp_path):
    """HMC columns and HMCV vectors written from the format model (pinned to
    the reference's readers by the host tests) read bit-exactly, through the
    type-specific readers and the qcd_getVector dispatcher"""
    cols = [orc.gaussian_spinor(L, 60 + k) for k in range(12)]
    lib = _vlib()
    geo = q.Geometry(L, TH)
    vec = q.Vector(geo)
    p = tmp_path / "prop.hmc"
    p.write_bytes(legacy_formats.hmc_file(cols, L))
    for nu in range(4):
        for c in range(3):
            vec.a[:] = 0
            fn = lib.qcd_getVectorHMC(str(p).encode(), nu, c, vec.ref) if (nu + c) % 2 else \
                lib.qcd_getVector(str(p).encode(), 1, nu, c, vec.ref)
            assert fn == 0
            assert np.array_equal(np.array(vec.a).reshape(cols[0].shape), cols[nu * 3 + c]), (nu, c)
    p.write_bytes(legacy_formats.hmcv_file(cols[7], L))
    for call in (lambda: lib.qcd_getVectorHMCV(str(p).encode(), 3, 2, vec.ref),
                 lambda: lib.qcd_getVector(str(p).encode(), 2, 0, 0, vec.ref)):
        vec.a[:] = 0
        assert call() == 0
        assert np.array_equal(np.array(vec.a).reshape(cols[0].shape), cols[7])
    vec.close()
    geo.close()


def test_legacy_header_whitespace_and_errors(gpu, orc, tmp_path):
    """whitespace bytes at the start of the data move the data offset as in
    the reference (fscanf's trailing newline); a header whose L or T differ
    from the geometry, a file shorter than the column, a missing file and an
    unknown type are errors"""
    cols = [orc.gaussian_spinor(L, 80 + k) for k in range(12)]
    cols[0][0, 0, 0, 0] = struct.unpack(">d", b"\x20\x0a" + b"\x11" * 6)[0]
    blob = legacy_formats.hmc_file(cols, L)
    p = tmp_path / "prop.hmc"
    p.write_bytes(blob)
    lib = _vlib()
    geo = q.Geometry(L, TH)
    vec = q.Vector(geo)
    assert lib.qcd_getVectorHMC(str(p).encode(), 1, 1, vec.ref) == 0
    want = legacy_formats.read_vector(blob, L, 4)
    assert np.array_equal(np.array(vec.a).reshape(want.shape), want, equal_nan=True)
    # the last column starts 2 bytes late and runs past the end of the file
    assert lib.qcd_getVectorHMC(str(p).encode(), 3, 2, vec.ref) == 1
    assert lib.qcd_getVector(str(p).encode(), 7, 0, 0, vec.ref) == 1
    assert lib.qcd_getVectorHMC(str(tmp_path / "missing").encode(), 0, 0, vec.ref) == 1
    assert lib.qcd_getVectorCMI(str(tmp_path / "missing").encode(), 0, 0, vec.ref) == 1
    for bad in ((4, 4, 6, 2), (8, 2, 6, 2)):
        g2 = q.Geometry(bad, TH)
        v2 = q.Vector(g2)
        p.write_bytes(legacy_formats.hmc_file([orc.gaussian_spinor(L, 1)] * 12, L))
        assert lib.qcd_getVectorHMC(str(p).encode(), 0, 0, v2.ref) == 1
        assert lib.qcd_getVectorHMCV(str(p).encode(), 0, 0, v2.ref) == 1
        v2.close()
        g2.close()
    p.write_bytes(legacy_formats.cmi_file(cols[1], L)[:-4])
    assert lib.qcd_getVectorCMI(str(p).encode(), 0, 0, vec.ref) == 1
    vec.close()
    geo.close()
