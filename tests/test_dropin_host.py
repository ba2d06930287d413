"""Host-side behaviour of the drop-in C ABI (no GPU needed): the library
loads, exports every declared symbol, keeps the qcd.h struct layout, builds
the reference's geometry tables and returns the reference's error codes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import qcd_gb300 as q

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "qcdgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    # function declarations, not the pointer-to-array members "(*D)[4][3]"
    names = set(re.findall(r"\b((?:qcd|qcdgpu)_\w+|gcr|bicgstab|cgnr)\s*\((?!\s*\*)", src))
    return sorted(n for n in names if not n.endswith("_s"))


def test_library_exports_every_declared_symbol(qlib):
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(qlib, n)]
    assert not missing, missing
    for n in q.DROPIN_SYMBOLS:
        assert n in names


def test_struct_layout_matches_reference(ref):
    assert C.sizeof(q.QcdGeometry) == ref.lib.ref_sizeof_geometry()
    assert C.sizeof(q.QcdVector) == ref.lib.ref_sizeof_vector()
    assert C.sizeof(q.QcdGaugeField) == ref.lib.ref_sizeof_gauge()


def test_struct_layout_offsets():
    # LP64 layout of include/qcd.h with int-sized MPI handles
    assert C.sizeof(q.QcdVector) == 88
    assert q.QcdGeometry.initialized.offset > q.QcdGeometry.requests.offset
    assert q.QcdGeometry.plus.offset % 8 == 0


@pytest.mark.parametrize("L", [(4, 4, 4, 4), (6, 4, 2, 8), (2, 2, 2, 2)])
def test_geometry_tables_match_reference(qlib, ref, L):
    th = (np.pi, 0.0, 0.0, 0.0)
    geo = q.Geometry(L, th)
    assert geo.ok
    s = geo.s
    V, V3 = geo.V, geo.V // L[0]
    t = ref.geometry(L, th)

    def arr(ptr, n):
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy()

    assert np.array_equal(arr(s.plus, 4 * V), t["plus"].ravel())
    assert np.array_equal(arr(s.minus, 4 * V), t["minus"].ravel())
    p3 = arr(s.plus3d, 4 * V3).reshape(V3, 4)[:, 1:]
    m3 = arr(s.minus3d, 4 * V3).reshape(V3, 4)[:, 1:]
    assert np.array_equal(p3, t["plus3d"][:, 1:])
    assert np.array_equal(m3, t["minus3d"][:, 1:])
    assert np.array_equal(arr(s.eo, V), t["eo"].ravel())
    assert s.edgePoints == len(t["edge"]) and np.array_equal(arr(s.edge, s.edgePoints), t["edge"])
    assert s.edge0Points == len(t["edge0"]) and np.array_equal(arr(s.edge0, s.edge0Points), t["edge0"])
    assert (s.V, s.V3, s.lV, s.lV3, s.nproc, s.initialized) == (V, V3, V, V3, 1, 1)
    assert list(s.theta) == list(th)
    geo.close()


def test_geometry_rejects_what_the_reference_rejects(qlib):
    assert q.Geometry((5, 4, 4, 4), P=(2, 1, 1, 1), nproc=2).rc == 1  # not divisible
    assert q.Geometry((3, 3, 3, 3)).rc == 1  # odd volume
    assert q.Geometry((1, 4, 4, 4)).rc == 1  # extent < 2
    # more than one process: one GPU holds the whole lattice
    assert q.Geometry((4, 4, 4, 4), P=(2, 1, 1, 1), nproc=2).rc == 1


def test_vectors_allocate_and_checks_run_without_gpu(qlib):
    geo = q.Geometry((4, 4, 4, 4))
    v, w = q.Vector(geo), q.Vector(geo)
    u = q.GaugeField(geo)
    v.a[:] = 1.0
    assert v.a.shape == (256, 4, 3, 2) and v.a.sum() == 256 * 24
    # uninitialised input vector: error 1 before any device work (qcd_wilson.c:139-143)
    bad = q.QcdVector()
    assert qlib.qcd_applyWilsonTMOp(w.ref, C.byref(bad), u.ref, -0.5, 0.0) == 1
    # uninitialised gauge field (:144-148)
    badu = q.QcdGaugeField()
    assert qlib.qcd_applyWilsonTMOp(w.ref, v.ref, C.byref(badu), -0.5, 0.0) == 1
    # in-place apply is rejected
    assert qlib.qcd_applyWilsonTMOp(v.ref, v.ref, u.ref, -0.5, 0.0) == 1
    # geometry mismatch (:149-166)
    geo2 = q.Geometry((4, 4, 4, 8))
    x = q.Vector(geo2)
    assert qlib.qcd_applyWilsonTMOp(w.ref, x.ref, u.ref, -0.5, 0.0) == 1
    # a halo "in flight" is refused as qcd_communication.c:25-29 does
    geo.s.numOfRequests = 2
    assert qlib.qcd_communicateVectorPMGaugeP(v.ref, u.ref) == 1
    qlib.qcd_waitall(C.byref(geo.s))
    assert geo.s.numOfRequests == 0
    assert qlib.qcd_communicateVectorPMGaugeP(v.ref, u.ref) == 0
    for o in (v, w, x, u):
        o.close()
    geo.close()
    geo2.close()


def test_server_result_layout_matches_the_header(tmp_path):
    """the ctypes mirror of qcdgpu_server_result has the C struct's size and
    field offsets (compiled from include/qcdgpu.h with gcc)"""
    import subprocess

    fields = [f[0] for f in q.ServerResult._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "qcdgpu.h"\nint main(void){\n'
                   ' printf("%zu", sizeof(qcdgpu_server_result));\n'
                   + "".join(f' printf(" %zu", offsetof(qcdgpu_server_result, {n}));\n' for n in fields)
                   + ' printf("\\n"); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=gnu99", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == C.sizeof(q.ServerResult)
    assert out[1:] == [getattr(q.ServerResult, n).offset for n in fields]


def test_c_program_links_against_the_library(qlib, tmp_path):
    """A qcd_lib-style C driver compiles against include/qcdgpu.h and links."""
    import subprocess

    src = tmp_path / "driver.c"
    src.write_text(
        '#include <stdio.h>\n#include <math.h>\n#include "qcdgpu.h"\n'
        "int main(void){ qcd_geometry geo; qcd_uint_2 L[4]={4,4,4,4}, P[4]={1,1,1,1};\n"
        " qcd_real_8 th[4]={M_PI,0,0,0}; qcd_vector v, Dv; qcd_gaugeField u;\n"
        " if(qcd_initGeometry(&geo,L,P,th,0,1)) return 2;\n"
        " if(qcd_initVector(&v,&geo)||qcd_initVector(&Dv,&geo)||qcd_initGaugeField(&u,&geo)) return 3;\n"
        " printf(\"%lu %lu\\n\", (unsigned long)geo.V, (unsigned long)sizeof(qcd_geometry));\n"
        " if(0) { qcd_applyWilsonTMOp(&Dv,&v,&u,-0.5,0.0); gcr(&Dv,&v,&u,0.15,0.0,32,&geo); }\n"
        " qcd_destroyVector(&v); qcd_destroyVector(&Dv); qcd_destroyGaugeField(&u); qcd_destroyGeometry(&geo); return 0; }\n")
    root = os.path.dirname(HEADER)
    exe = tmp_path / "driver"
    subprocess.run(["gcc", "-std=gnu99", "-I", root, str(src), "-o", str(exe), q.LIB_PATH, "-lm",
                    f"-Wl,-rpath,{os.path.dirname(q.LIB_PATH)}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split()[0] == "256"
    assert int(out.stdout.split()[1]) == C.sizeof(q.QcdGeometry)


def test_injected_allocation_failures_return_the_reference_error(qlib):
    """host-side fault injection: the drop-in's allocation failures return the
    reference's code 1 with its message (qcd_init.c:437-442, 614-665), leave
    nothing allocated, and the next allocation succeeds again"""
    lib = q.lib()
    lib.qcdgpu_inject_alloc_failures.argtypes = [C.c_int]
    geo = q.Geometry((4, 4, 4, 4))
    assert geo.ok
    try:
        assert lib.qcdgpu_inject_alloc_failures(2) == 0
        v = q.QcdVector()
        assert lib.qcd_initVector(C.byref(v), C.byref(geo.s)) == 1
        assert not v.initialized
        assert "qcd_initVector" in lib.qcdgpu_last_error().decode()
        assert "Out of memory" in lib.qcdgpu_last_error().decode()
        u = q.QcdGaugeField()
        assert lib.qcd_initGaugeField(C.byref(u), C.byref(geo.s)) == 1
        assert "qcd_initGaugeField" in lib.qcdgpu_last_error().decode()
        vec = q.Vector(geo)  # the injected failures are used up
        vec.a[:] = 1.0
        vec.close()
    finally:
        lib.qcdgpu_inject_alloc_failures(0)
        geo.close()


def _site_vectors(seed):
    rng = np.random.default_rng(seed)
    vec = rng.normal(size=(4, 3, 2))
    u = rng.normal(size=(3, 3, 2))
    return np.ascontiguousarray(vec), np.ascontiguousarray(u)


def test_site_helpers_match_reference(qlib, ref):
    """qcd_onePlusGamma / qcd_oneMinusGamma (mu = 0..5), qcd_applyU,
    qcd_applyUDagger, qcd_massTerms and qcd_phaseMul against the reference's
    own functions (lib/src/qcd_wilson.c:18-103) on the same inputs"""
    lib = q.lib()
    R = ref.lib
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    for n in ("qcd_onePlusGamma", "qcd_oneMinusGamma"):
        getattr(R, n).argtypes = [dp, dp, C.c_uint16]
    for n in ("qcd_applyU", "qcd_applyUDagger"):
        getattr(R, n).argtypes = [dp, dp, dp]
    R.qcd_massTerms.argtypes = [dp, dp, C.c_double, C.c_double]
    R.qcd_phaseMul.argtypes = [dp, q.QcdComplex16]
    for seed in range(3):
        vec, u = _site_vectors(seed)
        for mu in range(6):
            for n in ("qcd_onePlusGamma", "qcd_oneMinusGamma"):
                a, b = np.zeros_like(vec), np.zeros_like(vec)
                getattr(lib, n)(a, vec, mu)
                getattr(R, n)(b, vec, mu)
                assert np.array_equal(a, b), (n, mu)  # entries 0, +-1, +-i: exact
        for n in ("qcd_applyU", "qcd_applyUDagger"):
            a, b = np.zeros_like(vec), np.zeros_like(vec)
            getattr(lib, n)(a, u, vec)
            getattr(R, n)(b, u, vec)
            assert np.max(np.abs(a - b)) <= 1e-15 * np.max(np.abs(b)), n
        a, b = np.zeros_like(vec), np.zeros_like(vec)
        lib.qcd_massTerms(a, vec, 4.3, -0.27)
        R.qcd_massTerms(b, vec, 4.3, -0.27)
        assert np.max(np.abs(a - b)) <= 1e-15 * np.max(np.abs(b))
        a, b = vec.copy(), vec.copy()
        lib.qcd_phaseMul(a, q.QcdComplex16(0.6, -0.8))
        R.qcd_phaseMul(b, q.QcdComplex16(0.6, -0.8))
        assert np.max(np.abs(a - b)) <= 1e-15


def test_site_helpers_algebra(qlib):
    """the helpers against their definitions in the chiral basis (no reference
    needed): (1 +- gamma_mu), gamma_4 = -gamma_0, gamma_5 = diag(1, 1, -1, -1)"""
    G = np.zeros((6, 4, 4), dtype=complex)
    G[0][0, 2] = G[0][1, 3] = G[0][2, 0] = G[0][3, 1] = -1
    G[1][0, 3] = G[1][1, 2] = -1j
    G[1][2, 1] = G[1][3, 0] = 1j
    G[2][0, 3] = G[2][3, 0] = -1
    G[2][1, 2] = G[2][2, 1] = 1
    G[3][0, 2] = G[3][3, 1] = -1j
    G[3][1, 3] = G[3][2, 0] = 1j
    G[4] = -G[0]
    G[5] = np.diag([1, 1, -1, -1])
    lib = q.lib()
    vec, u = _site_vectors(9)
    vc = vec[..., 0] + 1j * vec[..., 1]
    uc = u[..., 0] + 1j * u[..., 1]

    def cx(a):
        return a[..., 0] + 1j * a[..., 1]

    for mu in range(6):
        a = np.zeros_like(vec)
        lib.qcd_onePlusGamma(a, vec, mu)
        assert np.allclose(cx(a), (np.eye(4) + G[mu]) @ vc, atol=1e-15)
        lib.qcd_oneMinusGamma(a, vec, mu)
        assert np.allclose(cx(a), (np.eye(4) - G[mu]) @ vc, atol=1e-15)
    a = np.zeros_like(vec)
    lib.qcd_applyU(a, u, vec)
    assert np.allclose(cx(a), vc @ uc.T, atol=1e-14)
    lib.qcd_applyUDagger(a, u, vec)
    assert np.allclose(cx(a), vc @ uc.conj(), atol=1e-14)
    lib.qcd_massTerms(a, vec, 4.3, -0.27)
    assert np.allclose(cx(a), 4.3 * vc + 1j * -0.27 * (G[5] @ vc), atol=1e-14)


@pytest.mark.parametrize("driver", ["invert", "b_minus_Dx"])
def test_reference_drivers_link_unmodified(qlib, tmp_path, driver):
    """the reference's own drivers, compiled unmodified against include/qcd.h
    (oracle/Makefile ref), link against the library with nothing else: every
    qcd_lib call they make is exported (invert.c keeps its own gcr())"""
    import subprocess

    from oracle.oracle import HERE

    obj = os.path.join(HERE, "_ref", f"{driver}_dropin.o")
    if not os.path.exists(obj):
        pytest.skip("reference drivers not built here (needs the reference source tree)")
    exe = tmp_path / driver
    out = subprocess.run(["gcc", obj, "-o", str(exe), q.LIB_PATH, "-lm"], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


PARAMS = (b"<processors_txyz>1 1 1 1</processors_txyz>\n<lattice_txyz>16 8 8 8</lattice_txyz>\n"
          b"<source_type>HMC_PROPAGATOR</source_type>\n<source>/data/prop.src</source>\n"
          b"<solution>/data/prop.src_inverted</solution>\n<cfg_name>/data/conf.2000</cfg_name>\n"
          b"<N_restart>32</N_restart>\n<kappa>0.160856</kappa>\n<mu>0.0085</mu>\n")
TAGS = ["<lattice_txyz>", "<source>", "<solution>", "<cfg_name>", "<N_restart>", "<kappa>", "<mu>",
        "<processors_txyz>"]


def _params(lib, path):
    lib.qcd_getParams.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    lib.qcd_getParams.restype = C.c_void_p
    lib.qcd_getParam.argtypes = [C.c_char_p, C.c_void_p, C.c_int]
    lib.qcd_getParam.restype = C.c_char_p
    n = C.c_int()
    buf = lib.qcd_getParams(str(path).encode(), C.byref(n))
    return buf, n.value


def test_parameter_file_parsing(qlib, tmp_path):
    """qcd_getParams / qcd_getParam (qcd_io.c:83-129): len = size + 1, values
    cut at the next '<', tags found in any order; a missing file is NULL"""
    p = tmp_path / "invert.ini"
    p.write_bytes(PARAMS)
    buf, n = _params(qlib, p)
    assert buf and n == len(PARAMS) + 1
    got = {t: qlib.qcd_getParam(t.encode(), buf, n) for t in TAGS}
    assert got["<lattice_txyz>"] == b"16 8 8 8" and got["<source>"] == b"/data/prop.src"
    assert got["<solution>"] == b"/data/prop.src_inverted" and got["<mu>"] == b"0.0085"
    assert got["<processors_txyz>"] == b"1 1 1 1"  # found after later tags were cut
    assert qlib.qcd_getParam(b"<absent>", buf, n) == b""
    assert _params(qlib, tmp_path / "missing.ini")[0] is None


def test_parameter_file_parsing_matches_reference(qlib, refio, tmp_path):
    """the same values as the reference's own qcd_getParams / qcd_getParam"""
    p = tmp_path / "invert.ini"
    p.write_bytes(PARAMS)
    mine, n = _params(qlib, p)
    theirs, m = _params(refio.lib, p)
    assert n == m
    for t in TAGS:
        assert qlib.qcd_getParam(t.encode(), mine, n) == refio.lib.qcd_getParam(t.encode(), theirs, m), t
