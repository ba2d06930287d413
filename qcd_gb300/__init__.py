"""qcd_gb300 -- Python access to the GB300 Wilson-twisted-mass library.

The library itself is ``_build/libqcdgpu.so`` (C ABI declared in
``include/qcdgpu.h``), built by :func:`qcd_gb300.build.build`. This module
mirrors its two interfaces:

* the qcd_lib drop-in (``qcd_initGeometry``, ``qcd_applyWilsonTMOp``,
  ``gcr`` ...) on ctypes copies of the ``qcd.h`` structs
  (:class:`Geometry`, :class:`Vector`, :class:`GaugeField`), whose data arrays
  are exposed as numpy views in the reference layout;
* the device API (``qcdgpu_*``): :class:`Field`, :class:`Gauge`,
  :func:`dslash`, :func:`solve`.

Importing never falls back to CPU arithmetic: if the shared library is
missing, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqcdgpu.so")

F64, F32, F16 = 0, 1, 2
OP_D, OP_Q, OP_DDAG, OP_DDAGD = 0, 1, 2, 3
ARITH_F64, ARITH_DF64 = 0, 1
SOLVER_GCR, SOLVER_BICGSTAB, SOLVER_CGNR, SOLVER_CGNR_EO, SOLVER_BICGSTABL_EO = 0, 1, 2, 3, 4

_u8p = C.POINTER(C.c_uint64)


class QcdGeometry(C.Structure):
    """include/qcd.h:44-87 (MPI handles int-sized)."""
    _fields_ = [
        ("V", C.c_uint64), ("V3", C.c_uint64), ("L", C.c_uint16 * 4),
        ("lV", C.c_uint64), ("lV3", C.c_uint64), ("lL", C.c_uint16 * 4), ("Pos", C.c_uint16 * 4),
        ("theta", C.c_double * 4), ("myid", C.c_uint32), ("nproc", C.c_uint32),
        ("Pplus", C.c_uint32 * 4), ("Pminus", C.c_uint32 * 4),
        ("plus", _u8p), ("minus", _u8p), ("plus3d", _u8p), ("minus3d", _u8p), ("eo", _u8p),
        ("startBminus", C.c_uint64 * 4), ("startBplus", C.c_uint64 * 4),
        ("startBminus3d", C.c_uint64 * 4), ("startBplus3d", C.c_uint64 * 4),
        ("boundarySize", C.c_uint64), ("boundarySize3d", C.c_uint64),
        ("edge", _u8p), ("edgePoints", C.c_uint64), ("edge0", _u8p), ("edge0Points", C.c_uint64),
        ("requests", C.c_int * 32), ("numOfRequests", C.c_int),
        ("stypeV", C.c_int * 4), ("rtypeV", C.c_int * 4), ("stypeU", C.c_int * 4),
        ("rtypeU", C.c_int * 4), ("stypeT", C.c_int * 4), ("rtypeT", C.c_int * 4),
        ("stypeP", C.c_int * 4), ("rtypeP", C.c_int * 4),
        ("initialized", C.c_uint16),
    ]


class QcdVector(C.Structure):
    """include/qcd.h:90-97."""
    _fields_ = [("D", C.c_void_p), ("Bplus", C.c_void_p * 4), ("Bminus", C.c_void_p * 4),
                ("geo", C.POINTER(QcdGeometry)), ("initialized", C.c_uint16)]


class QcdGaugeField(C.Structure):
    """include/qcd.h:119-126."""
    _fields_ = [("D", C.c_void_p), ("Bplus", C.c_void_p * 4), ("Bminus", C.c_void_p * 4),
                ("geo", C.POINTER(QcdGeometry)), ("initialized", C.c_uint16)]


class QcdComplex16(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class SolveParams(C.Structure):
    """qcdgpu_solve_params (include/qcdgpu.h)."""
    _fields_ = [("solver", C.c_int), ("op", C.c_int), ("inner_prec", C.c_int), ("tol", C.c_double),
                ("maxiter", C.c_int), ("restart", C.c_int), ("delta", C.c_double),
                ("iters", C.c_int), ("reliable_updates", C.c_int), ("true_residual", C.c_double),
                ("status", C.c_int)]


# every symbol include/qcdgpu.h declares (checked against the .so by the tests)
DROPIN_SYMBOLS = [
    "qcd_initGeometry", "qcd_destroyGeometry", "qcd_initVector", "qcd_destroyVector",
    "qcd_initGaugeField", "qcd_destroyGaugeField", "qcd_applyWilsonTMOp",
    "qcd_applyWilsonTMOpNoScripts", "qcd_applyWilsonTMOpNoOptim", "qcd_applyQTMOp",
    "qcd_zeroVector", "qcd_setVector", "qcd_copyVector", "qcd_mulVectorC", "qcd_scaleVector",
    "qcd_subVector", "qcd_addVector", "qcd_axpyVector", "qcd_mulAdjointVectorVector",
    "qcd_normVector", "qcd_gamma5Vector", "qcd_communicateVectorPMGaugeP", "qcd_waitall",
    "qcd_onePlusGamma", "qcd_oneMinusGamma", "qcd_applyU", "qcd_applyUDagger", "qcd_massTerms", "qcd_phaseMul",
    "qcd_z2Vector", "qcd_getVectorCMI", "qcd_getVectorHMC", "qcd_getVectorHMCV", "qcd_getVector",
    "qcd_writeVectorCMI", "qcd_writeVector", "qcd_getParams", "qcd_getParam",
    "gcr", "bicgstab", "cgnr",
]

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built; run qcd_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    gp, vp, up = C.POINTER(QcdGeometry), C.POINTER(QcdVector), C.POINTER(QcdGaugeField)
    L.qcd_initGeometry.argtypes = [gp, C.POINTER(C.c_uint16), C.POINTER(C.c_uint16), C.POINTER(C.c_double), C.c_int, C.c_int]
    L.qcd_destroyGeometry.argtypes = [gp]
    L.qcd_initVector.argtypes = [vp, gp]
    L.qcd_destroyVector.argtypes = [vp]
    L.qcd_initGaugeField.argtypes = [up, gp]
    L.qcd_destroyGaugeField.argtypes = [up]
    for n in ("qcd_applyWilsonTMOp", "qcd_applyWilsonTMOpNoScripts", "qcd_applyWilsonTMOpNoOptim", "qcd_applyQTMOp"):
        getattr(L, n).argtypes = [vp, vp, up, C.c_double, C.c_double]
    L.qcd_zeroVector.argtypes = [vp]
    L.qcd_setVector.argtypes = [vp, QcdComplex16]
    L.qcd_copyVector.argtypes = [vp, vp]
    L.qcd_mulVectorC.argtypes = [vp, QcdComplex16]
    L.qcd_scaleVector.argtypes = [vp, C.c_double]
    L.qcd_subVector.argtypes = [vp, vp, vp]
    L.qcd_addVector.argtypes = [vp, vp, vp]
    L.qcd_axpyVector.argtypes = [vp, QcdComplex16, vp, vp]
    L.qcd_mulAdjointVectorVector.argtypes = [vp, vp]
    L.qcd_mulAdjointVectorVector.restype = QcdComplex16
    L.qcd_normVector.argtypes = [vp]
    L.qcd_normVector.restype = C.c_double
    L.qcd_gamma5Vector.argtypes = [vp]
    L.qcd_communicateVectorPMGaugeP.argtypes = [vp, up]
    L.qcd_waitall.argtypes = [gp]
    L.gcr.argtypes = [vp, vp, up, C.c_double, C.c_double, C.c_uint32, gp]
    L.bicgstab.argtypes = [vp, vp, up, C.c_double, C.c_double, C.c_double, C.c_uint32, gp]
    L.cgnr.argtypes = [vp, vp, up, C.c_double, C.c_double, C.c_double, C.c_uint32, gp]
    L.qcdgpu_last_error.restype = C.c_char_p
    L.qcdgpu_set_stream.argtypes = [C.c_void_p]
    L.qcdgpu_set_gcr_compat.argtypes = [C.c_int]
    L.qcdgpu_set_gcr_compat.restype = None
    L.qcdgpu_set_f64_arith.argtypes = [C.c_int]
    L.qcdgpu_kernel_launches.restype = C.c_uint64
    for n in ("qcdgpu_vector_make_resident", "qcdgpu_vector_to_host", "qcdgpu_vector_to_device", "qcdgpu_vector_release"):
        getattr(L, n).argtypes = [vp]
    L.qcdgpu_gauge_upload.argtypes = [up]
    L.qcdgpu_gauge_release.argtypes = [up]
    vpp = C.POINTER(C.c_void_p)
    L.qcdgpu_gauge_create.argtypes = [vpp, _ip, _dp, C.c_int]
    L.qcdgpu_gauge_destroy.argtypes = [C.c_void_p]
    L.qcdgpu_gauge_load.argtypes = [C.c_void_p, _dp]
    L.qcdgpu_gauge_store.argtypes = [C.c_void_p, _dp]
    L.qcdgpu_gauge_convert.argtypes = [C.c_void_p, C.c_void_p]
    L.qcdgpu_gauge_synthetic.argtypes = [C.c_void_p, C.c_uint64, C.c_double]
    L.qcdgpu_gauge_recon.argtypes = [C.c_void_p]
    L.qcdgpu_gauge_bytes.argtypes = [C.c_void_p]
    L.qcdgpu_gauge_bytes.restype = C.c_size_t
    L.qcdgpu_plaquette.argtypes = [C.c_void_p]
    L.qcdgpu_plaquette.restype = C.c_double
    L.qcdgpu_field_create.argtypes = [vpp, _ip, C.c_int]
    L.qcdgpu_field_destroy.argtypes = [C.c_void_p]
    L.qcdgpu_field_load.argtypes = [C.c_void_p, _dp]
    L.qcdgpu_field_store.argtypes = [C.c_void_p, _dp]
    L.qcdgpu_field_copy.argtypes = [C.c_void_p, C.c_void_p]
    L.qcdgpu_field_gaussian.argtypes = [C.c_void_p, C.c_uint64]
    L.qcdgpu_field_point.argtypes = [C.c_void_p, _ip, C.c_int, C.c_int]
    L.qcdgpu_measure_fma_rate.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.qcdgpu_field_noise.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_int]
    L.qcd_z2Vector.argtypes = [vp, C.c_int]
    L.qcd_z2Vector.restype = None
    L.qcdgpu_set_noise_seed.argtypes = [C.c_uint64]
    for n in ("qcd_onePlusGamma", "qcd_oneMinusGamma"):
        getattr(L, n).argtypes = [_dp, _dp, C.c_uint16]
        getattr(L, n).restype = None
    for n in ("qcd_applyU", "qcd_applyUDagger"):
        getattr(L, n).argtypes = [_dp, _dp, _dp]
        getattr(L, n).restype = None
    L.qcd_massTerms.argtypes = [_dp, _dp, C.c_double, C.c_double]
    L.qcd_massTerms.restype = None
    L.qcd_phaseMul.argtypes = [_dp, QcdComplex16]
    L.qcd_phaseMul.restype = None
    L.qcdgpu_field_bytes.argtypes = [C.c_void_p]
    L.qcdgpu_field_bytes.restype = C.c_size_t
    L.qcdgpu_field_data.argtypes = [C.c_void_p]
    L.qcdgpu_field_data.restype = C.c_void_p
    L.qcdgpu_dslash.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int]
    L.qcdgpu_axpy.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    L.qcdgpu_norm2.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    L.qcdgpu_dot.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    L.qcdgpu_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.POINTER(SolveParams)]
    L.qcdgpu_dot_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    L.qcdgpu_mfield_create.argtypes = [vpp, _ip, C.c_int]
    L.qcdgpu_mfield_destroy.argtypes = [C.c_void_p]
    L.qcdgpu_mfield_set.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    L.qcdgpu_mfield_get.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.qcdgpu_dslash_mrhs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int]
    L.qcdgpu_twop_proton.argtypes = [C.c_void_p, C.c_void_p, _ip, C.c_int, C.c_int, _ip, C.c_int, _dp]
    L.qcd_apeSmear3d.argtypes = [up, up, C.c_double]
    L.qcd_gaussIteration3d.argtypes = [vp, up, C.c_double, C.c_uint32]
    L.qcd_calculatePlaquette.argtypes = [up]
    L.qcd_calculatePlaquette.restype = C.c_double
    L.qcdgpu_gauge_ape3d.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int]
    L.qcdgpu_field_gauss3d.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int]
    L.qcdgpu_smeared_source.argtypes = [C.c_void_p, C.c_void_p, _ip, C.c_int, C.c_int, C.c_double, C.c_int,
                                        C.c_double, C.c_int]
    L.qcdgpu_set_mrhs_variant.argtypes = [C.c_int]
    L.qcdgpu_mrhs_tuned.argtypes = [_ip, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.qcdgpu_mrhs_tc_timeouts.argtypes = [C.POINTER(C.c_uint)]
    L.qcdgpu_mrhs_tc_test_hook.argtypes = [C.c_int, C.c_int]
    L.qcdgpu_server_create.argtypes = [vpp, C.c_size_t, C.c_int]
    L.qcdgpu_server_destroy.argtypes = [C.c_void_p]
    L.qcdgpu_server_add_gauge.argtypes = [C.c_void_p, C.c_void_p]
    L.qcdgpu_server_submit.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_uint64, C.c_double, C.c_double,
                                       C.c_int, C.c_double, C.c_int, C.c_int]
    L.qcdgpu_server_progress.argtypes = [C.c_void_p]
    L.qcdgpu_server_poll.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.qcdgpu_server_fetch.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.qcdgpu_server_release.argtypes = [C.c_void_p, C.c_int]
    L.qcdgpu_server_stats.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.qcdgpu_batch_create.argtypes = [vpp, C.c_void_p, C.c_int]
    L.qcdgpu_batch_create_eo.argtypes = [vpp, C.c_void_p, C.c_int]
    L.qcdgpu_batch_destroy.argtypes = [C.c_void_p]
    L.qcdgpu_batch_add.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_double,
                                   C.c_int, C.c_double, C.c_int]
    L.qcdgpu_batch_step.argtypes = [C.c_void_p, C.c_int]
    L.qcdgpu_batch_active.argtypes = [C.c_void_p]
    L.qcdgpu_batch_free_slots.argtypes = [C.c_void_p]
    L.qcdgpu_batch_poll.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, C.c_int]
    L.qcdgpu_batch_bytes.argtypes = [C.c_void_p]
    L.qcdgpu_batch_bytes.restype = C.c_size_t
    _lib = L
    return L


class QcdGpuError(RuntimeError):
    pass


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise QcdGpuError(f"{what} failed: {lib().qcdgpu_last_error().decode()}")


def volume(L) -> int:
    return int(L[0]) * int(L[1]) * int(L[2]) * int(L[3])


# --------------------------------------------------------------- drop-in
class Geometry:
    """A qcd_geometry built by the library's qcd_initGeometry (one rank)."""

    def __init__(self, L, theta=(np.pi, 0.0, 0.0, 0.0), P=(1, 1, 1, 1), myid=0, nproc=1):
        self.s = QcdGeometry()
        self.L = tuple(int(x) for x in L)
        Ls = (C.c_uint16 * 4)(*self.L)
        Ps = (C.c_uint16 * 4)(*P)
        th = (C.c_double * 4)(*theta)
        self.rc = lib().qcd_initGeometry(C.byref(self.s), Ls, Ps, th, myid, nproc)
        self.ok = self.rc == 0

    @property
    def V(self) -> int:
        return volume(self.L)

    def close(self):
        if self.ok:
            lib().qcd_destroyGeometry(C.byref(self.s))
            self.ok = False


class Vector:
    """qcd_vector allocated by qcd_initVector; ``a`` is a numpy view of D."""

    def __init__(self, geo: Geometry):
        self.geo = geo
        self.s = QcdVector()
        _check(lib().qcd_initVector(C.byref(self.s), C.byref(geo.s)), "qcd_initVector")
        buf = (C.c_double * (geo.V * 24)).from_address(self.s.D)
        self.a = np.ctypeslib.as_array(buf).reshape(geo.V, 4, 3, 2)

    @property
    def ref(self):
        return C.byref(self.s)

    def close(self):
        if self.s.initialized:
            lib().qcd_destroyVector(C.byref(self.s))
            self.s.initialized = 0


class GaugeField:
    """qcd_gaugeField allocated by qcd_initGaugeField; ``a`` is a numpy view of D."""

    def __init__(self, geo: Geometry):
        self.geo = geo
        self.s = QcdGaugeField()
        _check(lib().qcd_initGaugeField(C.byref(self.s), C.byref(geo.s)), "qcd_initGaugeField")
        buf = (C.c_double * (geo.V * 72)).from_address(self.s.D)
        self.a = np.ctypeslib.as_array(buf).reshape(geo.V, 4, 3, 3, 2)

    @property
    def ref(self):
        return C.byref(self.s)

    def close(self):
        if self.s.initialized:
            lib().qcd_destroyGaugeField(C.byref(self.s))
            self.s.initialized = 0


# ----------------------------------------------------------- device API
class Field:
    """Device spinor field (qcdgpu_field)."""

    def __init__(self, L, prec=F64):
        self.L = np.ascontiguousarray(L, dtype=np.int32)
        self.prec = prec
        h = C.c_void_p()
        _check(lib().qcdgpu_field_create(C.byref(h), self.L, prec), "qcdgpu_field_create")
        self.h = h

    @property
    def V(self) -> int:
        return volume(self.L)

    def load(self, arr: np.ndarray) -> "Field":
        _check(lib().qcdgpu_field_load(self.h, np.ascontiguousarray(arr, dtype=np.float64)), "field_load")
        return self

    def store(self) -> np.ndarray:
        out = np.empty((self.V, 4, 3, 2))
        _check(lib().qcdgpu_field_store(self.h, out), "field_store")
        return out

    def gaussian(self, seed: int) -> "Field":
        _check(lib().qcdgpu_field_gaussian(self.h, seed), "field_gaussian")
        return self

    def noise(self, seed: int, t_slice: int = -1, kind: int = 4) -> "Field":
        """Z4 (kind 4) or Z2 (kind 2) noise on time-slice t_slice (all sites when negative)"""
        _check(lib().qcdgpu_field_noise(self.h, seed, t_slice, kind), "field_noise")
        return self

    def point(self, x, spin, colour) -> "Field":
        _check(lib().qcdgpu_field_point(self.h, np.ascontiguousarray(x, dtype=np.int32), spin, colour), "field_point")
        return self

    def copy_from(self, other: "Field") -> "Field":
        _check(lib().qcdgpu_field_copy(self.h, other.h), "field_copy")
        return self

    def norm2(self) -> float:
        r = C.c_double()
        _check(lib().qcdgpu_norm2(self.h, C.byref(r)), "norm2")
        return r.value

    def dot(self, other: "Field") -> complex:
        r = (C.c_double * 2)()
        _check(lib().qcdgpu_dot(self.h, other.h, r), "dot")
        return complex(r[0], r[1])

    @property
    def nbytes(self) -> int:
        return lib().qcdgpu_field_bytes(self.h)

    def close(self):
        if self.h:
            lib().qcdgpu_field_destroy(self.h)
            self.h = None


class Gauge:
    """Device gauge field (qcdgpu_gauge)."""

    def __init__(self, L, theta=(np.pi, 0.0, 0.0, 0.0), prec=F64):
        self.L = np.ascontiguousarray(L, dtype=np.int32)
        self.theta = np.ascontiguousarray(theta, dtype=np.float64)
        self.prec = prec
        h = C.c_void_p()
        _check(lib().qcdgpu_gauge_create(C.byref(h), self.L, self.theta, prec), "qcdgpu_gauge_create")
        self.h = h

    def load(self, arr: np.ndarray) -> "Gauge":
        _check(lib().qcdgpu_gauge_load(self.h, np.ascontiguousarray(arr, dtype=np.float64)), "gauge_load")
        return self

    def store(self) -> np.ndarray:
        out = np.empty((volume(self.L), 4, 3, 3, 2))
        _check(lib().qcdgpu_gauge_store(self.h, out), "gauge_store")
        return out

    def synthetic(self, seed: int, eps: float) -> "Gauge":
        _check(lib().qcdgpu_gauge_synthetic(self.h, seed, eps), "gauge_synthetic")
        return self

    def convert_from(self, other: "Gauge") -> "Gauge":
        _check(lib().qcdgpu_gauge_convert(self.h, other.h), "gauge_convert")
        return self

    @property
    def recon(self) -> int:
        return lib().qcdgpu_gauge_recon(self.h)

    @property
    def nbytes(self) -> int:
        return lib().qcdgpu_gauge_bytes(self.h)

    def plaquette(self) -> float:
        return lib().qcdgpu_plaquette(self.h)

    def close(self):
        if self.h:
            lib().qcdgpu_gauge_destroy(self.h)
            self.h = None


def dslash(out: Field, inp: Field, g: Gauge, kappa: float, mu: float = 0.0, op: int = OP_D, arith: int = -1):
    _check(lib().qcdgpu_dslash(out.h, inp.h, g.h, kappa, mu, op, arith), "qcdgpu_dslash")


def axpy(out: Field, a: complex, x: Field, y: Field):
    _check(lib().qcdgpu_axpy(out.h, a.real, a.imag, x.h, y.h), "qcdgpu_axpy")


def solve(x: Field, b: Field, g: Gauge, kappa: float, mu: float = 0.0, solver=SOLVER_CGNR, op=OP_D,
          inner_prec=F64, tol=1e-10, maxiter=100000, restart=32, delta=0.1) -> SolveParams:
    p = SolveParams(solver=solver, op=op, inner_prec=inner_prec, tol=tol, maxiter=maxiter,
                    restart=restart, delta=delta)
    rc = lib().qcdgpu_solve(x.h, b.h, g.h, kappa, mu, C.byref(p))
    if rc == 3:
        raise QcdGpuError(f"qcdgpu_solve failed: {lib().qcdgpu_last_error().decode()}")
    return p


def release_work() -> None:
    """free the solvers' pooled work fields"""
    lib().qcdgpu_release_work()


def set_stream(stream_ptr: int | None):
    _check(lib().qcdgpu_set_stream(C.c_void_p(stream_ptr or 0)), "set_stream")


def sync():
    _check(lib().qcdgpu_sync(), "sync")


def kernel_launches() -> int:
    return lib().qcdgpu_kernel_launches()


class MField:
    """Multi-RHS device field (qcdgpu_mfield): up to 64 FP16 spinors."""

    def __init__(self, L, nrhs):
        self.L = np.ascontiguousarray(L, dtype=np.int32)
        self.n = nrhs
        h = C.c_void_p()
        _check(lib().qcdgpu_mfield_create(C.byref(h), self.L, nrhs), "qcdgpu_mfield_create")
        self.h = h

    def set(self, r: int, f: Field) -> "MField":
        _check(lib().qcdgpu_mfield_set(self.h, r, f.h), "mfield_set")
        return self

    def get(self, r: int, f: Field) -> Field:
        _check(lib().qcdgpu_mfield_get(f.h, self.h, r), "mfield_get")
        return f

    def close(self):
        if self.h:
            lib().qcdgpu_mfield_destroy(self.h)
            self.h = None


def ape3d(out: "Gauge", inp: "Gauge", alpha: float, n: int = 1) -> "Gauge":
    """n 3D APE smearing steps out <- inp (device FP64 gauge fields)."""
    _check(lib().qcdgpu_gauge_ape3d(out.h, inp.h, alpha, n), "qcdgpu_gauge_ape3d")
    return out


def gauss3d(v: "Field", g: "Gauge", alpha: float, t: int, n: int = 1) -> "Field":
    """n 3D Gaussian smearing steps of v on time-slice t."""
    _check(lib().qcdgpu_field_gauss3d(v.h, g.h, alpha, t, n), "qcdgpu_field_gauss3d")
    return v


def smeared_source(f: "Field", g: "Gauge", x, spin: int, colour: int, ape_alpha: float = 0.5, ape_n: int = 20,
                   gauss_alpha: float = 4.0, gauss_n: int = 50) -> "Field":
    """point source at x = (t, x, y, z), Gaussian-smeared on APE-smeared links."""
    _check(lib().qcdgpu_smeared_source(f.h, g.h, np.ascontiguousarray(x, dtype=np.int32), spin, colour, ape_alpha,
                                       ape_n, gauss_alpha, gauss_n), "qcdgpu_smeared_source")
    return f


def twop_proton(up, dn, xsrc, t0: int, t1: int, moms) -> np.ndarray:
    """proton two-point function of twop.c on 12 + 12 FP64 propagator columns
    (Field, column nu * 3 + c2); returns corr[t - t0, j] (complex)."""
    moms = np.ascontiguousarray(moms, dtype=np.int32).reshape(-1, 3)
    cu = (C.c_void_p * 12)(*[f.h.value for f in up])
    cd = (C.c_void_p * 12)(*[f.h.value for f in dn])
    out = np.zeros((t1 - t0 + 1) * len(moms) * 2)
    _check(lib().qcdgpu_twop_proton(C.cast(cu, C.c_void_p), C.cast(cd, C.c_void_p),
                                    np.ascontiguousarray(xsrc, dtype=np.int32), t0, t1, moms, len(moms), out),
           "qcdgpu_twop_proton")
    out = out.reshape(t1 - t0 + 1, len(moms), 2)
    return out[..., 0] + 1j * out[..., 1]


def set_mrhs_variant(v: int) -> None:
    """-1: tuned; 1: tensor-core kernel; 64 / 128 / 256: SIMT kernel with that block size."""
    _check(lib().qcdgpu_set_mrhs_variant(v), "qcdgpu_set_mrhs_variant")


def mrhs_tuned(L, nrhs):
    """(variant, threads) the tuner chose for this volume and slot count, or None."""
    v, t = C.c_int(), C.c_int()
    if lib().qcdgpu_mrhs_tuned(np.asarray(L, np.int32), nrhs, C.byref(v), C.byref(t)) != 0:
        return None
    return ("simt" if v.value == 0 else "mma", t.value)


def dslash_mrhs(out: MField, inp: MField, g: Gauge, kappa: float, mu: float = 0.0, op: int = OP_D, nact=None):
    _check(lib().qcdgpu_dslash_mrhs(out.h, inp.h, g.h, kappa, mu, op, inp.n if nact is None else nact),
           "qcdgpu_dslash_mrhs")


class Batch:
    """Batched multi-RHS solver with continuous admission (qcdgpu_batch)."""

    def __init__(self, g: Gauge, capacity: int, eo: bool = False):
        """eo: solve each system through its even/odd Schur complement."""
        self.h = C.c_void_p()
        self.capacity = capacity
        create = lib().qcdgpu_batch_create_eo if eo else lib().qcdgpu_batch_create
        _check(create(C.byref(self.h), g.h, capacity), "qcdgpu_batch_create")

    def add(self, x: Field, b: Field, kappa: float, mu: float = 0.0, op: int = OP_D, tol: float = 1e-10,
            maxiter: int = 0, delta: float = 0.1, tag: int = 0) -> int:
        """Returns the slot, or -1 when the batch is full."""
        k = lib().qcdgpu_batch_add(self.h, x.h, b.h, kappa, mu, op, tol, maxiter, delta, tag)
        if k == -2:
            raise QcdGpuError(f"qcdgpu_batch_add failed: {lib().qcdgpu_last_error().decode()}")
        return k

    def step(self, iterations: int = 16) -> None:
        if lib().qcdgpu_batch_step(self.h, iterations) != 0:
            raise QcdGpuError(f"qcdgpu_batch_step failed: {lib().qcdgpu_last_error().decode()}")

    @property
    def active(self) -> int:
        return lib().qcdgpu_batch_active(self.h)

    @property
    def free_slots(self) -> int:
        return lib().qcdgpu_batch_free_slots(self.h)

    def nbytes(self) -> int:
        return lib().qcdgpu_batch_bytes(self.h)

    def poll(self, max_n: int = 64):
        """[(tag, status, iterations, true_residual)] of the retired right-hand sides."""
        tags = np.zeros(max_n, np.int32)
        st = np.zeros(max_n, np.int32)
        it = np.zeros(max_n, np.int32)
        tr = np.zeros(max_n, np.float64)
        n = lib().qcdgpu_batch_poll(self.h, tags, st, it, tr, max_n)
        return [(int(tags[i]), int(st[i]), int(it[i]), float(tr[i])) for i in range(n)]

    def close(self):
        if self.h:
            lib().qcdgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerResult(C.Structure):
    _fields_ = [("tag", C.c_int), ("status", C.c_int), ("nrhs", C.c_int), ("max_iters", C.c_int),
                ("max_true_residual", C.c_double), ("queue_s", C.c_double), ("latency_s", C.c_double),
                ("total_iters", C.c_int)]


class Server:
    """Request server with continuous batching and HBM-budget admission (qcdgpu_server)."""

    def __init__(self, hbm_budget_bytes: int, slots: int = 32):
        self.h = C.c_void_p()
        _check(lib().qcdgpu_server_create(C.byref(self.h), int(hbm_budget_bytes), slots), "qcdgpu_server_create")

    def add_gauge(self, g: Gauge) -> int:
        gid = lib().qcdgpu_server_add_gauge(self.h, g.h)
        if gid < 0:
            raise QcdGpuError(f"qcdgpu_server_add_gauge failed: {lib().qcdgpu_last_error().decode()}")
        return gid

    def submit(self, gauge_id: int, nrhs: int, kappa: float, mu: float = 0.0, op: int = OP_D, tol: float = 1e-10,
               tag: int = 0, sources=None, seed: int = 0, maxiter: int = 0) -> None:
        src = None
        if sources is not None:
            arr = (C.c_void_p * nrhs)(*[f.h.value for f in sources])
            src = C.cast(arr, C.c_void_p)
        _check(lib().qcdgpu_server_submit(self.h, gauge_id, nrhs, src, seed, kappa, mu, op, tol, maxiter, tag),
               "qcdgpu_server_submit")

    def progress(self) -> None:
        _check(lib().qcdgpu_server_progress(self.h), "qcdgpu_server_progress")

    def poll(self, max_n: int = 256):
        out = (ServerResult * max_n)()
        n = lib().qcdgpu_server_poll(self.h, C.cast(out, C.c_void_p), max_n)
        return [dict(tag=r.tag, status=r.status, nrhs=r.nrhs, max_iters=r.max_iters,
                     max_true_residual=r.max_true_residual, queue_s=r.queue_s, latency_s=r.latency_s,
                     total_iters=r.total_iters)
                for r in out[:n]]

    def fetch(self, tag: int, col: int, dst: Field) -> Field:
        _check(lib().qcdgpu_server_fetch(self.h, tag, col, dst.h), "qcdgpu_server_fetch")
        return dst

    def release(self, tag: int) -> None:
        _check(lib().qcdgpu_server_release(self.h, tag), "qcdgpu_server_release")

    def stats(self):
        used, queued, active = C.c_size_t(), C.c_int(), C.c_int()
        _check(lib().qcdgpu_server_stats(self.h, C.byref(used), C.byref(queued), C.byref(active)),
               "qcdgpu_server_stats")
        return dict(bytes_used=used.value, queued=queued.value, active_rhs=active.value)

    def close(self):
        if self.h:
            lib().qcdgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
