"""The file formats pinned to the reference's own readers and writers
(lib/src/qcd_io.c compiled unmodified, oracle/_ref/libqcdio.so), no GPU.

The Python format models (tests/lime_util.py, tests/legacy_formats.py) that
the GPU file tests build their inputs and expectations from are checked here
against the reference: files the models write are read by qcd_io.c's readers,
and files qcd_io.c's writers produce (committed as tests/golden/io_L4235.npz
by tests/golden/make_io_golden.py) parse to the models' records and bytes.
The golden checks need no reference library; the reader checks skip without
it.
"""
import struct

import numpy as np
import pytest

from tests import legacy_formats as lf
from tests import lime_util
from tests.conftest import EPS_PLAQ_060

L = (8, 4, 6, 2)


def as_bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


# ------------------------------------------------- files the reference wrote
def test_reference_written_gauge_file_matches_the_model(golden):
    g = golden["io_L4235"]
    Lg = tuple(int(x) for x in g["L"])
    recs = lime_util.parse(g["conf_lime"].tobytes())
    assert [(r[0], r[1], r[2]) for r in recs] == [("ildg-format", True, False), ("xlf-info", False, False),
                                                  ("ildg-binary-data", False, True)]
    assert b"<precision> 64 </precision>" in recs[0][3]
    assert b"<lx> 2 </lx>" in recs[0][3] and b"<lt> 4 </lt>" in recs[0][3]
    assert recs[1][3] == g["message"].tobytes()
    assert recs[2][3] == lime_util.ildg_payload(g["u"], Lg, 64)


@pytest.mark.parametrize("key,kind", [("prop_lime", "propagator"), ("source_lime", "source")])
def test_reference_written_vector_files_match_the_model(golden, key, kind):
    g = golden["io_L4235"]
    Lg = tuple(int(x) for x in g["L"])
    recs = lime_util.parse(g[key].tobytes())
    assert [r[0] for r in recs] == [f"{kind}-type", f"etmc-{kind}-format", "scidac-binary-data"]
    assert recs[0][3] == (b"DiracFermion_Sink" if kind == "propagator" else b"DiracFermion_Source")
    assert b"<precision>64</precision>" in recs[1][3]
    assert recs[2][3] == lime_util.etmc_payload(g["v"], Lg, 64)


def test_reference_written_cmi_file_matches_the_model(golden):
    g = golden["io_L4235"]
    assert g["vec_cmi"].tobytes() == lf.cmi_file(g["v"], tuple(int(x) for x in g["L"]))


# ------------------------------------------- files the models wrote, read by
# the reference
def test_ildg_gauge_from_the_model_reads_back(refio, orc, tmp_path):
    u = orc.gauge_synthetic(L, 51, EPS_PLAQ_060)
    p = tmp_path / "conf.lime"
    p.write_bytes(lime_util.ildg_file(u, L, 64))
    rc, got = refio.get_gauge(p, L)
    assert rc == 0 and np.array_equal(got, u)
    rc, _ = refio.get_gauge(tmp_path / "missing.lime", L)
    assert rc == 1


def test_fp32_ildg_reference_swaps_only_the_first_time_slice(refio, orc, tmp_path):
    """qcd_getGaugeLime's FP32 branch byte-swaps 2*4*3*3*lV3 floats
    (qcd_io.c:377, the spatial volume, not lV) on a little-endian host: the
    t = 0 slice reads correctly, every other slice keeps big-endian bytes.
    The GPU library swaps the whole payload (its FP32 test expects the
    file's values everywhere); this pins the reference's behaviour so the
    difference is a known one."""
    u = orc.gauge_synthetic(L, 51, EPS_PLAQ_060)
    p = tmp_path / "conf.lime"
    p.write_bytes(lime_util.ildg_file(u, L, 32))
    rc, got = refio.get_gauge(p, L)
    assert rc == 0
    want = u.astype(np.float32).astype(np.float64)
    Lt, Lx, Ly, Lz = L
    G = got.reshape(Lz, Ly, Lx, Lt, -1)
    W = want.reshape(Lz, Ly, Lx, Lt, -1)
    assert np.array_equal(G[:, :, :, 0], W[:, :, :, 0])
    with np.errstate(invalid="ignore"):  # some swapped words are NaNs
        unswapped = want.astype(np.float32).view(np.uint32).byteswap().view(np.float32).astype(np.float64)
    U = unswapped.reshape(Lz, Ly, Lx, Lt, -1)
    assert np.array_equal(G[:, :, :, 1:], U[:, :, :, 1:], equal_nan=True)


@pytest.mark.parametrize("prec", [64, 32])
def test_etmc_vector_from_the_model_reads_back(refio, orc, tmp_path, prec):
    v = orc.gaussian_spinor(L, 53)
    p = tmp_path / "prop.lime"
    p.write_bytes(lime_util.etmc_file(v, L, prec))
    rc, got = refio.get_vector(p, L, refio.PROP_LIME)
    want = v if prec == 64 else v.astype(np.float32).astype(np.float64)
    assert rc == 0 and np.array_equal(got, want)


def test_cmi_vector_from_the_model_reads_back(refio, orc, tmp_path):
    """CMI ignores the source column (qcd_io.c:907-982): one vector per file"""
    v = orc.gaussian_spinor(L, 54)
    p = tmp_path / "vec.cmi"
    p.write_bytes(lf.cmi_file(v, L))
    for nu, c in ((0, 0), (3, 2)):
        rc, got = refio.get_vector(p, L, refio.CMI, nu, c)
        assert rc == 0 and np.array_equal(got, v.astype(np.float32).astype(np.float64))


def test_hmc_columns_and_hmcv_from_the_model_read_back(refio, orc, tmp_path):
    cols = [orc.gaussian_spinor(L, 60 + k) for k in range(12)]
    p = tmp_path / "prop.hmc"
    p.write_bytes(lf.hmc_file(cols, L))
    for nu in range(4):
        for c in range(3):
            rc, got = refio.get_vector(p, L, refio.HMC, nu, c)
            assert rc == 0 and np.array_equal(got, cols[nu * 3 + c]), (nu, c)
    p.write_bytes(lf.hmcv_file(cols[5], L))
    rc, got = refio.get_vector(p, L, refio.HMCV, 2, 1)  # HMCV ignores the column
    assert rc == 0 and np.array_equal(got, cols[5])


def test_hmc_header_whitespace_quirk(refio, orc, tmp_path):
    """fscanf's trailing "\\n" also swallows whitespace bytes at the start of
    the binary data, so the reference reads from a shifted offset; the model
    (legacy_formats.read_vector) reproduces that, and the GPU tests hold the
    library to the model."""
    cols = [orc.gaussian_spinor(L, 80 + k) for k in range(12)]
    cols[0][0, 0, 0, 0] = struct.unpack(">d", b"\x20\x0a" + b"\x11" * 6)[0]
    blob = lf.hmc_file(cols, L)
    assert lf.data_offset(blob) == blob.index(b"\n") + 3
    p = tmp_path / "prop.hmc"
    p.write_bytes(blob)
    rc, got = refio.get_vector(p, L, refio.HMC, 1, 1)
    assert rc == 0
    assert np.array_equal(as_bits(got), as_bits(lf.read_vector(blob, L, 4)))
    assert not np.array_equal(got, cols[4])


def test_hmc_dimension_check_and_errors(refio, orc, tmp_path):
    """the header's L and T must match geo L[1] and L[0] (qcd_io.c:1228-1233);
    a missing file and an unknown type fail"""
    cols = [orc.gaussian_spinor(L, 90 + k) for k in range(12)]
    p = tmp_path / "prop.hmc"
    p.write_bytes(lf.hmc_file(cols, L))
    for bad in ((4, 4, 6, 2), (8, 2, 6, 2)):
        assert refio.get_vector(p, bad, refio.HMC)[0] == 1
        assert refio.get_vector(p, bad, refio.HMCV)[0] == 1
    assert refio.get_vector(tmp_path / "missing", L, refio.HMC)[0] == 1
    assert refio.get_vector(tmp_path / "missing", L, refio.CMI)[0] == 1
    assert refio.get_vector(p, L, 7)[0] == 1
