"""ctypes access to the CPU oracle.

TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
baseline leg of the benchmark use this module as the checker; the GPU
library never imports it.

Two libraries:

* ``Oracle`` -- the C restatement (``qcd_oracle.c``), built on any machine;
* ``Reference`` -- the reference's own sources compiled unmodified
  (``_ref/libqcdref.so``); present only where the reference tree was
  available at build time;
* ``ReferenceIO`` -- the reference's file readers and writers
  (``lib/src/qcd_io.c``) compiled unmodified (``_ref/libqcdio.so``), with a
  single-rank MPI-IO stand-in and the LIME container restated from its
  published format (``lime_format.c``; c-lime is not in the reference tree).

All arrays use the reference host layout: spinors ``float64[V, 4, 3, 2]``,
gauge fields ``float64[V, 4, 3, 3, 2]`` with site ``t + Lt*(x + Lx*(y + Ly*z))``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libqcdref.so")
REF_IO_SO = os.path.join(HERE, "_ref", "libqcdio.so")
# where the reference's source tree lies, for `make ref`: the build entry
# point passes it (environment variable QCD_REFERENCE_TREE)
REF_TREE_ENV = "QCD_REFERENCE_TREE"

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(with_ref: bool | None = None, ref_tree: str | None = None) -> None:
    """Compile the restatement and, when a reference source tree is given
    (``ref_tree`` or $QCD_REFERENCE_TREE) and exists, the reference."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_tree = ref_tree or os.environ.get(REF_TREE_ENV)
    if with_ref is None:
        with_ref = bool(ref_tree) and os.path.isdir(ref_tree)
    if with_ref:
        if not ref_tree:
            raise RuntimeError(f"building the reference needs its source tree (${REF_TREE_ENV})")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_tree}"], check=True)


def _L(L):
    return np.ascontiguousarray(L, dtype=np.int32)


def _th(theta):
    return np.ascontiguousarray(theta, dtype=np.float64)


def volume(L) -> int:
    return int(L[0]) * int(L[1]) * int(L[2]) * int(L[3])


class Oracle:
    """The C restatement of the reference path."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(with_ref=False)
        lib = C.CDLL(path)
        self.lib = lib
        for name in ("orc_dslash", "orc_qop", "orc_dslash_dag"):
            f = getattr(lib, name)
            f.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double]
            f.restype = None
        lib.orc_dslash_fast.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double]
        lib.orc_dslash_fast.restype = C.c_int
        lib.orc_gamma5.argtypes = [_dp, _dp, C.c_size_t]
        lib.orc_norm.argtypes = [_dp, C.c_size_t]
        lib.orc_norm.restype = C.c_double
        lib.orc_dot.argtypes = [_dp, _dp, _dp, C.c_size_t]
        lib.orc_axpy.argtypes = [_dp, C.c_double, C.c_double, _dp, _dp, C.c_size_t]
        lib.orc_scale.argtypes = [_dp, _dp, C.c_double, C.c_size_t]
        lib.orc_mulc.argtypes = [_dp, _dp, C.c_double, C.c_double, C.c_size_t]
        lib.orc_add.argtypes = [_dp, _dp, _dp, C.c_size_t]
        lib.orc_sub.argtypes = [_dp, _dp, _dp, C.c_size_t]
        lib.orc_gcr.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double, C.c_int, C.c_int]
        lib.orc_gcr.restype = C.c_int
        lib.orc_invert_gcr.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double, C.c_int,
                                       C.c_int, C.c_double, C.c_int, C.POINTER(C.c_double)]
        lib.orc_invert_gcr.restype = C.c_int
        lib.orc_bicgstab.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double, C.c_int,
                                     C.c_double, C.c_int, C.POINTER(C.c_double)]
        lib.orc_bicgstab.restype = C.c_int
        lib.orc_cgnr.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double,
                                 C.c_double, C.c_int, C.POINTER(C.c_double)]
        lib.orc_cgnr.restype = C.c_int
        lib.orc_true_residual.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double, C.c_int]
        lib.orc_true_residual.restype = C.c_double
        lib.orc_exp_iM.argtypes = [_dp]
        lib.orc_project_su3.argtypes = [_dp]
        lib.orc_plaquette.argtypes = [_dp, _ip]
        lib.orc_plaquette.restype = C.c_double
        lib.orc_ape3d.argtypes = [_dp, _dp, _ip, C.c_double]
        lib.orc_gauss3d.argtypes = [_dp, _dp, _ip, C.c_double, C.c_int]
        lib.orc_rng_bits.argtypes = [C.c_uint64, C.c_uint64]
        lib.orc_rng_bits.restype = C.c_uint64
        lib.orc_gauss.argtypes = [C.c_uint64, C.c_uint64]
        lib.orc_gauss.restype = C.c_double
        lib.orc_gaussian_spinor.argtypes = [_dp, C.c_size_t, C.c_uint64]
        lib.orc_z4_spinor.argtypes = [_dp, C.c_size_t, C.c_uint64]
        lib.orc_noise_spinor.argtypes = [_dp, _ip, C.c_uint64, C.c_int, C.c_int]
        lib.orc_gauge_synthetic.argtypes = [_dp, _ip, C.c_uint64, C.c_double]
        lib.orc_gauge_unit.argtypes = [_dp, C.c_size_t]
        lib.orc_twop_proton.argtypes = [_dp, _dp, _ip, _ip, C.c_int, C.c_int, _ip, C.c_int, _dp]
        lib.orc_twop_tables.argtypes = [_dp, _dp, _dp]

    # --- operator -------------------------------------------------------
    def dslash(self, v, u, L, theta, kappa=None, m=None, tm=0.0, op="D"):
        if m is None:
            m = 1.0 / (2.0 * kappa) - 4.0
        out = np.empty_like(v)
        f = {"D": self.lib.orc_dslash, "Q": self.lib.orc_qop, "Ddag": self.lib.orc_dslash_dag}[op]
        f(out, np.ascontiguousarray(v), np.ascontiguousarray(u), _L(L), _th(theta), m, tm)
        return out

    def dslash_fast(self, v, u, L, theta, kappa=None, m=None, tm=0.0, out=None):
        """D v by the timed CPU baseline (qcd_cpu_timing.c: the reference's
        half-spinor algorithm at -O3); not the parity checker"""
        if m is None:
            m = 1.0 / (2.0 * kappa) - 4.0
        if out is None:
            out = np.empty_like(v)
        rc = self.lib.orc_dslash_fast(out, v, u, _L(L), _th(theta), m, tm)
        if rc != 0:
            raise MemoryError("orc_dslash_fast: neighbour tables not allocated")
        return out

    def gamma5(self, v):
        out = np.empty_like(v)
        self.lib.orc_gamma5(out, np.ascontiguousarray(v), v.shape[0])
        return out

    # --- BLAS -------------------------------------------------------------
    def norm(self, v):
        return self.lib.orc_norm(np.ascontiguousarray(v), v.shape[0])

    def dot(self, a, b):
        r = np.zeros(2)
        self.lib.orc_dot(r, np.ascontiguousarray(a), np.ascontiguousarray(b), a.shape[0])
        return complex(r[0], r[1])

    def axpy(self, a, x, y):
        out = np.empty_like(x)
        self.lib.orc_axpy(out, a.real, a.imag, np.ascontiguousarray(x), np.ascontiguousarray(y), x.shape[0])
        return out

    # --- solvers ------------------------------------------------------------
    def gcr(self, src, u, L, theta, kappa, mu, n, fixed=True):
        sol = np.empty_like(src)
        rc = self.lib.orc_gcr(sol, src, u, _L(L), _th(theta), kappa, mu, n, int(fixed))
        return sol, rc

    def invert_gcr(self, src, u, L, theta, kappa, mu, n, fixed=True, maxres=1e-8, maxiter=10000):
        sol = np.empty_like(src)
        rr = C.c_double()
        it = self.lib.orc_invert_gcr(sol, src, u, _L(L), _th(theta), kappa, mu, n, int(fixed),
                                     maxres, maxiter, C.byref(rr))
        return sol, it, rr.value

    def bicgstab(self, b, u, L, theta, kappa, mu=0.0, op="D", tol=1e-10, maxiter=10000):
        x = np.empty_like(b)
        rr = C.c_double()
        it = self.lib.orc_bicgstab(x, np.ascontiguousarray(b), u, _L(L), _th(theta), kappa, mu,
                                   {"D": 0, "Q": 1}[op], tol, maxiter, C.byref(rr))
        return x, it, rr.value

    def cgnr(self, b, u, L, theta, kappa, mu=0.0, tol=1e-10, maxiter=10000):
        x = np.empty_like(b)
        rr = C.c_double()
        it = self.lib.orc_cgnr(x, np.ascontiguousarray(b), u, _L(L), _th(theta), kappa, mu, tol,
                               maxiter, C.byref(rr))
        return x, it, rr.value

    def true_residual(self, x, b, u, L, theta, kappa, mu=0.0, op="D"):
        return self.lib.orc_true_residual(np.ascontiguousarray(x), np.ascontiguousarray(b), u,
                                          _L(L), _th(theta), kappa, mu, {"D": 0, "Q": 1}[op])

    # --- contractions ---------------------------------------------------------
    def twop_proton(self, up, dn, L, xsrc, t0, t1, moms):
        """proton two-point function of twop.c: corr[t - t0, j] (complex). The
        propagators (V, 4, 4, 3, 3, 2) are copied (the oracle phases them in place)."""
        up = np.array(up, dtype=np.float64, copy=True, order="C")
        dn = np.array(dn, dtype=np.float64, copy=True, order="C")
        moms = np.ascontiguousarray(moms, dtype=np.int32).reshape(-1, 3)
        corr = np.zeros((t1 - t0 + 1, len(moms), 2))
        self.lib.orc_twop_proton(up, dn, _L(L), np.ascontiguousarray(xsrc, dtype=np.int32), t0, t1, moms,
                                 len(moms), corr)
        return corr[..., 0] + 1j * corr[..., 1]

    def twop_tables(self):
        cg5, bcg5, p13 = np.zeros((4, 4)), np.zeros((4, 4)), np.zeros((4, 4, 2))
        self.lib.orc_twop_tables(cg5, bcg5, p13)
        return cg5, bcg5, p13[..., 0] + 1j * p13[..., 1]

    # --- setup ----------------------------------------------------------------
    def exp_iM(self, M):
        M = np.array(M, dtype=np.float64, copy=True).reshape(3, 3, 2)
        self.lib.orc_exp_iM(M)
        return M

    def project_su3(self, g):
        g = np.array(g, dtype=np.float64, copy=True).reshape(3, 3, 2)
        self.lib.orc_project_su3(g)
        return g

    def plaquette(self, u, L):
        return self.lib.orc_plaquette(np.ascontiguousarray(u), _L(L))

    def ape3d(self, u, L, alpha):
        out = np.empty_like(u)
        self.lib.orc_ape3d(out, np.ascontiguousarray(u), _L(L), alpha)
        return out

    def gauss3d(self, v, u, L, alpha, t):
        v = np.array(v, copy=True)
        self.lib.orc_gauss3d(v, np.ascontiguousarray(u), _L(L), alpha, t)
        return v

    def rng_bits(self, seed, ctr):
        return self.lib.orc_rng_bits(seed, ctr)

    def gaussian_spinor(self, L, seed):
        v = np.empty((volume(L), 4, 3, 2))
        self.lib.orc_gaussian_spinor(v, volume(L), seed)
        return v

    def noise_spinor(self, L, seed, t_slice=-1, kind=4):
        v = np.empty((volume(L), 4, 3, 2))
        self.lib.orc_noise_spinor(v, _L(L), seed, t_slice, kind)
        return v

    def z4_spinor(self, L, seed):
        v = np.empty((volume(L), 4, 3, 2))
        self.lib.orc_z4_spinor(v, volume(L), seed)
        return v

    def gauge_synthetic(self, L, seed, eps):
        u = np.empty((volume(L), 4, 3, 3, 2))
        self.lib.orc_gauge_synthetic(u, _L(L), seed, eps)
        return u

    def gauge_unit(self, L):
        u = np.empty((volume(L), 4, 3, 3, 2))
        self.lib.orc_gauge_unit(u, volume(L))
        return u


class Reference:
    """The reference library itself (compiled unmodified); single rank."""

    VARIANTS = {"TMOp": 0, "NoOptim": 1, "NoScripts": 2, "Q": 3}

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_SO)

    def __init__(self, path: str = REF_SO):
        lib = C.CDLL(path)
        self.lib = lib
        lib.ref_dslash.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double, C.c_int, C.c_int]
        lib.ref_dslash.restype = C.c_int
        lib.ref_gcr.argtypes = [_dp, _dp, _dp, _ip, _dp, C.c_double, C.c_double, C.c_int]
        lib.ref_gcr.restype = C.c_int
        lib.ref_blas.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, _ip, _dp]
        lib.ref_blas.restype = C.c_int
        lib.ref_plaquette.argtypes = [_dp, _ip]
        lib.ref_plaquette.restype = C.c_double
        lib.ref_ape3d.argtypes = [_dp, _dp, _ip, C.c_double]
        lib.ref_ape3d.restype = C.c_int
        lib.ref_gauss3d.argtypes = [_dp, _dp, _ip, C.c_double, C.c_int]
        lib.ref_gauss3d.restype = C.c_int
        lib.ref_exp_iM.argtypes = [_dp]
        lib.ref_project_su3.argtypes = [_dp]
        for n in ("ref_sizeof_geometry", "ref_sizeof_vector", "ref_sizeof_gauge"):
            getattr(lib, n).restype = C.c_size_t
        lib.ref_io_set.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_twop.argtypes = [C.c_char_p]
        lib.ref_twop.restype = C.c_int

    def dslash(self, v, u, L, theta, kappa=None, m=None, tm=0.0, variant="TMOp", reps=1):
        if m is None:
            m = 1.0 / (2.0 * kappa) - 4.0
        out = np.zeros_like(v)
        rc = self.lib.ref_dslash(out, np.ascontiguousarray(v), np.ascontiguousarray(u), _L(L),
                                 _th(theta), m, tm, self.VARIANTS[variant], reps)
        assert rc == 0
        return out

    def gcr(self, src, u, L, theta, kappa, mu, n):
        sol = np.zeros_like(src)
        rc = self.lib.ref_gcr(sol, np.ascontiguousarray(src), np.ascontiguousarray(u), _L(L),
                              _th(theta), kappa, mu, n)
        return sol, rc

    def blas(self, op, out, a, b, c=0j, L=None):
        res = np.zeros(2)
        self.lib.ref_blas(op, out, a, b, c.real, c.imag, _L(L), res)
        return res

    def plaquette(self, u, L):
        return self.lib.ref_plaquette(np.ascontiguousarray(u), _L(L))

    def ape3d(self, u, L, alpha):
        out = np.zeros_like(u)
        assert self.lib.ref_ape3d(out, np.ascontiguousarray(u), _L(L), alpha) == 0
        return out

    def gauss3d(self, v, u, L, alpha, t):
        v = np.array(v, copy=True)
        assert self.lib.ref_gauss3d(v, np.ascontiguousarray(u), _L(L), alpha, t) == 0
        return v

    def exp_iM(self, M):
        M = np.array(M, dtype=np.float64, copy=True).reshape(3, 3, 2)
        self.lib.ref_exp_iM(M)
        return M

    def project_su3(self, g):
        g = np.array(g, dtype=np.float64, copy=True).reshape(3, 3, 2)
        self.lib.ref_project_su3(g)
        return g

    def twop(self, u, up, dn, L, xsrc, t0, t1, moms, nsmear=0, alpha=4.0, nape=0, alpha_ape=0.5):
        """runs the reference's twop.c main() on in-memory inputs (propagators
        (V, 4, 4, 3, 3, 2), links (V, 4, 3, 3, 2)); returns corr[t - t0, j]"""
        import tempfile

        moms = np.asarray(moms, dtype=int).reshape(-1, 3)
        with tempfile.TemporaryDirectory() as d:
            mfile, cfile = os.path.join(d, "mom.txt"), os.path.join(d, "corr.dat")
            with open(mfile, "w") as f:
                f.write(f"{len(moms)}\n" + "".join(f"{a} {b} {c}\n" for a, b, c in moms))
            params = (f"<processors_txyz>1 1 1 1</processors_txyz><lattice_txyz>{L[0]} {L[1]} {L[2]} {L[3]}"
                      f"</lattice_txyz><t>{t0} {t1}</t><source_pos_txyz>{xsrc[0]} {xsrc[1]} {xsrc[2]} {xsrc[3]}"
                      f"</source_pos_txyz><propagator_u>up</propagator_u><propagator_d>down</propagator_d>"
                      f"<cfg_name>conf</cfg_name><corr_name>{cfile}</corr_name><momenta_list>{mfile}"
                      f"</momenta_list><alpha_gauss>{alpha!r}</alpha_gauss><nsmear_gauss>{nsmear}</nsmear_gauss>"
                      f"<alpha_APE>{alpha_ape!r}</alpha_APE><nsmear_APE>{nape}</nsmear_APE>").encode()
            keep = [np.ascontiguousarray(u, dtype=np.float64), np.ascontiguousarray(up, dtype=np.float64),
                    np.ascontiguousarray(dn, dtype=np.float64)]
            self.lib.ref_io_set(params, *[a.ctypes.data for a in keep])
            assert self.lib.ref_twop(b"params.txt") == 0
            self.lib.ref_io_set(None, None, None, None)
            rows = np.loadtxt(cfile, ndmin=2)
        corr = np.zeros((t1 - t0 + 1, len(moms)), dtype=complex)
        for k, row in enumerate(rows):
            corr[k // len(moms), k % len(moms)] = row[4] + 1j * row[5]
        return corr

    def twop_tables(self):
        """qcd_CGAMMA[5], qcd_BAR_CGAMMA[5] and PROJECTOR[13] as compiled"""
        c16 = C.c_double * (6 * 4 * 4 * 2)
        cg = np.frombuffer(c16.in_dll(self.lib, "qcd_CGAMMA"), dtype=np.float64).reshape(6, 4, 4, 2)
        bcg = np.frombuffer(c16.in_dll(self.lib, "qcd_BAR_CGAMMA"), dtype=np.float64).reshape(6, 4, 4, 2)
        pr = np.frombuffer((C.c_double * (25 * 16 * 2)).in_dll(self.lib, "PROJECTOR"), dtype=np.float64)
        pr = pr.reshape(25, 4, 4, 2)
        return (cg[5, ..., 0] + 1j * cg[5, ..., 1], bcg[5, ..., 0] + 1j * bcg[5, ..., 1],
                pr[13, ..., 0] + 1j * pr[13, ..., 1])

    def geometry(self, L, theta=(0, 0, 0, 0)):
        """neighbour tables, even/odd list and edge lists of qcd_initGeometry"""
        V = volume(L)
        V3 = V // int(L[0])
        u64 = np.uint64
        t = dict(plus=np.zeros((V, 4), u64), minus=np.zeros((V, 4), u64),
                 plus3d=np.zeros((V3, 4), u64), minus3d=np.zeros((V3, 4), u64),
                 eo=np.zeros((V // 2, 2), u64), edge=np.zeros(V, u64), edge0=np.zeros(V3, u64))
        counts = np.zeros(4, u64)
        up = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
        self.lib.ref_geometry.argtypes = [_ip, _dp] + [up] * 8
        assert self.lib.ref_geometry(_L(L), _th(theta), t["plus"], t["minus"], t["plus3d"], t["minus3d"],
                                     t["eo"], t["edge"], t["edge0"], counts) == 0
        t["edge"] = t["edge"][: int(counts[0])]
        t["edge0"] = t["edge0"][: int(counts[1])]
        return t


def site_rel_err(a, b):
    """max over sites of |a(x) - b(x)| / |b(x)| (per-site relative norm)."""
    V = a.shape[0]
    d = np.linalg.norm((a - b).reshape(V, -1), axis=1)
    n = np.linalg.norm(b.reshape(V, -1), axis=1)
    return float(np.max(d / np.where(n > 0, n, 1.0)))


class ReferenceIO:
    """The reference's own qcd_io.c readers and writers; single rank.
    Vectors are float64[V, 4, 3, 2], gauge fields float64[V, 4, 3, 3, 2]."""

    CMI, HMC, HMCV, PROP_LIME, SOURCE_LIME = 0, 1, 2, 3, 4

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_IO_SO)

    def __init__(self, path: str = REF_IO_SO):
        lib = C.CDLL(path)
        self.lib = lib
        lib.refio_get_vector.argtypes = [_dp, C.c_char_p, _ip, C.c_int, C.c_int, C.c_int]
        lib.refio_write_vector.argtypes = [_dp, C.c_char_p, _ip, C.c_int, C.c_int, C.c_int]
        lib.refio_get_gauge.argtypes = [_dp, C.c_char_p, _ip]
        lib.refio_write_gauge.argtypes = [_dp, C.c_char_p, _ip, C.c_char_p]
        for n in ("refio_get_vector", "refio_write_vector", "refio_get_gauge", "refio_write_gauge"):
            getattr(lib, n).restype = C.c_int

    def get_vector(self, path, L, type_, nu=0, c2=0):
        """(rc, vector); qcd_getVector (qcd_io.c:1386)"""
        v = np.zeros((volume(L), 4, 3, 2))
        rc = self.lib.refio_get_vector(v, os.fsencode(path), _L(L), type_, nu, c2)
        return rc, v

    def write_vector(self, v, path, L, type_, nu=0, c2=0) -> int:
        """qcd_writeVector (qcd_io.c:1951): CMI or LIME"""
        return self.lib.refio_write_vector(np.ascontiguousarray(v, dtype=np.float64), os.fsencode(path), _L(L),
                                           type_, nu, c2)

    def get_gauge(self, path, L):
        """(rc, gauge); qcd_getGaugeField type qcd_GF_LIME (qcd_io.c:401)"""
        u = np.zeros((volume(L), 4, 3, 3, 2))
        rc = self.lib.refio_get_gauge(u, os.fsencode(path), _L(L))
        return rc, u

    def write_gauge(self, u, path, L, message="") -> int:
        """qcd_writeGaugeLime (qcd_io.c:421)"""
        return self.lib.refio_write_gauge(np.ascontiguousarray(u, dtype=np.float64), os.fsencode(path), _L(L),
                                          message.encode())
