"""Parity at the lattices the benchmark runs, against the CPU oracle.

The small-lattice tests pin every kernel to the reference's own outputs; these
repeat the comparison where the benchmark measures, because large lattices are
where index arithmetic (32-bit site indices, block strides, slab offsets) would
break first:

* 24^3 x 48 (663,552 sites, the single-RHS operator's benchmark): the
  float-float FP64 operator (D, D^+, Q, with and without twisted mass) and the
  native FP64 operator at <= 1e-13 relative per-site norm; FP32 and FP16
  storage at their usual bars; the FP64 true residual of an even/odd
  mixed-precision solve recomputed by the oracle (b_minus_Dx.c:152-172).
* 48^3 x 96 (10,616,832 sites, the multi-RHS benchmark): one FP64 apply at
  1e-13, the FP16 single-RHS apply and two multi-RHS slots against the oracle
  at 4e-3, every other slot against the FP64 GPU operator pinned in the same
  test, and one even/odd batch slot's FP64 true residual recomputed by the
  oracle.

The 48^3 x 96 tests hold ~25 GB of host memory and ~60 GB of device memory;
each oracle apply at that size takes ~15 s on one host core.
"""
import numpy as np
import pytest

import qcd_gb300 as q
from oracle.oracle import site_rel_err
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
TOL64 = 1e-13
L24 = (48, 24, 24, 24)
L48 = (96, 48, 48, 48)
TH = (np.pi, 0.0, 0.0, 0.0)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def bench24(gpu, orc):
    """the benchmark's 24^3 x 48 inputs: links built by the oracle's seeded recipe"""
    u = orc.gauge_synthetic(L24, 1000, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L24, 2000)
    g = q.Gauge(L24, TH).load(u)
    yield u, v, g
    g.close()


@pytest.mark.parametrize("tm", [0.0, 0.07])
def test_float_float_operator_24x48_vs_oracle(bench24, orc, tm):
    u, v, g = bench24
    fin, fout = q.Field(L24).load(v), q.Field(L24)
    for op, o in ((q.OP_D, "D"), (q.OP_DDAG, "Ddag"), (q.OP_Q, "Q")):
        q.dslash(fout, fin, g, 0.15, tm, op, q.ARITH_DF64)
        err = site_rel_err(fout.store(), orc.dslash(v, u, L24, TH, kappa=0.15, tm=tm, op=o))
        assert err <= TOL64, (o, err)
    fin.close()
    fout.close()


def test_native_fp64_and_low_precision_operators_24x48_vs_oracle(bench24, orc):
    u, v, g = bench24
    ref = orc.dslash(v, u, L24, TH, kappa=0.15, tm=0.05)
    fin, fout = q.Field(L24).load(v), q.Field(L24)
    q.dslash(fout, fin, g, 0.15, 0.05, q.OP_D, q.ARITH_F64)
    assert site_rel_err(fout.store(), ref) <= TOL64
    for prec, tol in ((q.F32, 2e-6), (q.F16, 4e-3)):
        gl = q.Gauge(L24, TH, prec).convert_from(g)
        fi, fo = q.Field(L24, prec).copy_from(fin), q.Field(L24, prec)
        q.dslash(fo, fi, gl, 0.15, 0.05, q.OP_D)
        assert rel(fout.copy_from(fo).store(), ref) <= tol, prec
        for f in (gl, fi, fo):
            f.close()
    fin.close()
    fout.close()


def test_even_odd_solve_24x48_true_residual_by_oracle(bench24, orc):
    """the benchmark's point-source solve: its FP64 true residual recomputed on
    the CPU (not by the library's own operator)"""
    u, _, g = bench24
    V = int(np.prod(L24))
    bh = np.zeros((V, 4, 3, 2))
    bh[0, 0, 0, 0] = 1.0
    b, x = q.Field(L24).load(bh), q.Field(L24)
    p = q.solve(x, b, g, 0.15, 0.0, solver=q.SOLVER_CGNR_EO, inner_prec=q.F16, tol=1e-10)
    assert p.status == 0
    res = orc.true_residual(x.store(), bh, u, L24, TH, 0.15)
    assert res <= 1e-10
    assert abs(res - p.true_residual) <= 1e-3 * 1e-10 + 1e-15
    b.close()
    x.close()


@pytest.fixture(scope="module")
def bench48(gpu):
    """48^3 x 96 links from the library's synthetic generator (the same seeded
    recipe as the oracle's, which small-lattice tests pin), copied to the host
    for the oracle"""
    g = q.Gauge(L48, TH).synthetic(3, EPS_PLAQ_060)
    u = g.store()
    yield u, g
    g.close()


def test_operators_48x96_vs_oracle(bench48, orc):
    """FP64 (float-float), FP16 single-RHS and the multi-RHS operator at
    10.6 M sites: slots 0 and 7 against the oracle, every slot against the
    FP64 GPU apply of the same spinor"""
    u, g = bench48
    nrhs = 8
    f = q.Field(L48).gaussian(500)
    v0 = f.store()
    ref0 = orc.dslash(v0, u, L48, TH, kappa=0.15, tm=0.03)
    fo = q.Field(L48)
    q.dslash(fo, f, g, 0.15, 0.03, q.OP_D, q.ARITH_DF64)
    assert site_rel_err(fo.store(), ref0) <= TOL64
    g16 = q.Gauge(L48, TH, q.F16).convert_from(g)
    fi16, fo16 = q.Field(L48, q.F16).copy_from(f), q.Field(L48, q.F16)
    q.dslash(fo16, fi16, g16, 0.15, 0.03, q.OP_D)
    assert rel(fo.copy_from(fo16).store(), ref0) <= 4e-3
    for x in (g16, fi16, fo16):
        x.close()
    mi, mo = q.MField(L48, nrhs), q.MField(L48, nrhs)
    for r in range(nrhs):
        mi.set(r, f.gaussian(500 + r))
    q.dslash_mrhs(mo, mi, g, 0.15, 0.03, q.OP_D, nrhs)
    ref7 = orc.dslash(f.gaussian(507).store(), u, L48, TH, kappa=0.15, tm=0.03)
    assert rel(mo.get(0, fo).store(), ref0) <= 4e-3
    assert rel(mo.get(7, fo).store(), ref7) <= 4e-3
    ff = q.Field(L48)
    for r in range(1, nrhs - 1):
        q.dslash(ff, f.gaussian(500 + r), g, 0.15, 0.03, q.OP_D, q.ARITH_DF64)
        assert rel(mo.get(r, fo).store(), ff.store()) <= 4e-3, r
    for x in (mi, mo, f, fo, ff):
        x.close()


def test_even_odd_batch_48x96_true_residual_by_oracle(bench48, orc):
    """one slot of a 4-slot even/odd batch at 48^3 x 96 (point sources at two
    positions) solved to 1e-10; the FP64 true residual recomputed on the CPU"""
    u, g = bench48
    V = int(np.prod(L48))
    srcs, xs = [], []
    for c in range(4):
        srcs.append(q.Field(L48).point(((c // 2) * L48[0] // 2, 0, 0, 0), c % 2, c % 3))
        xs.append(q.Field(L48))
    batch = q.Batch(g, 4, eo=True)
    for c in range(4):
        assert batch.add(xs[c], srcs[c], 0.15, 0.0, q.OP_D, tol=1e-10, maxiter=40000, tag=c) >= 0
    done = []
    while batch.active:
        batch.step(16)
        done += batch.poll()
    done += batch.poll()
    assert sorted(d[0] for d in done) == [0, 1, 2, 3] and all(d[1] == 0 for d in done)
    c = 3
    bh = np.zeros((V, 4, 3, 2))
    bh[(L48[0] // 2), c % 2, c % 3, 0] = 1.0  # site (t = 48, x = y = z = 0)
    res = orc.true_residual(xs[c].store(), bh, u, L48, TH, 0.15)
    assert res <= 1e-10
    assert abs(res - [d[3] for d in done if d[0] == c][0]) <= 1e-3 * 1e-10 + 1e-15
    batch.close()
    for x in srcs + xs:
        x.close()
