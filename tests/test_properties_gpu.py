"""Size-independent properties of the FP64 operator on the GPU (both the
native and the float-float kernel): free-field plane waves with the per-hop
boundary phase, gauge covariance, gamma_5-hermiticity, the unit-field
plaquette -- on small lattices and, for the cheap ones, on the 24^3 x 48
bench lattice."""
import numpy as np
import pytest

import qcd_gb300 as q
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu

# chiral basis of qcd_lib (lib/src/qcd_gamma.c:46-103), gamma_0..3 and gamma_5
G = np.zeros((5, 4, 4), dtype=complex)
G[0][0, 2] = G[0][1, 3] = G[0][2, 0] = G[0][3, 1] = -1
G[1][0, 3] = G[1][1, 2] = -1j
G[1][2, 1] = G[1][3, 0] = 1j
G[2][0, 3] = G[2][3, 0] = -1
G[2][1, 2] = G[2][2, 1] = 1
G[3][0, 2] = G[3][3, 1] = -1j
G[3][1, 3] = G[3][2, 0] = 1j
G[4] = np.diag([1, 1, -1, -1])


def cplx(a):
    return a[..., 0] + 1j * a[..., 1]


def real(c):
    return np.stack([c.real, c.imag], axis=-1)


def coords(L):
    V = int(np.prod(L))
    idx = np.arange(V)
    t = idx % L[0]
    x = (idx // L[0]) % L[1]
    y = (idx // (L[0] * L[1])) % L[2]
    z = idx // (L[0] * L[1] * L[2])
    return np.stack([t, x, y, z], axis=1)


@pytest.mark.parametrize("arith", [q.ARITH_F64, q.ARITH_DF64])
def test_free_field_plane_wave(gpu, orc, arith):
    L, th, kappa, mu = (8, 4, 6, 4), (np.pi, 0.3, 0.0, -0.5), 0.13, 0.07
    n = np.array([3, 1, -2, 1])
    p = (2 * np.pi * n + np.array(th)) / np.array(L)
    rng = np.random.default_rng(3)
    u0 = rng.normal(size=(4, 3)) + 1j * rng.normal(size=(4, 3))
    ph = np.exp(1j * (coords(L) @ (2 * np.pi * n / np.array(L))))
    psi = ph[:, None, None] * u0[None]
    M = (1 / (2 * kappa)) * np.eye(4) - np.sum(np.cos(p)) * np.eye(4) + 1j * mu * G[4]
    for m in range(4):
        M = M + 1j * np.sin(p[m]) * G[m]
    want = ph[:, None, None] * (M @ u0)[None]
    g = q.Gauge(L, th).load(orc.gauge_unit(L))
    fi, fo = q.Field(L).load(real(psi)), q.Field(L)
    q.dslash(fo, fi, g, kappa, mu, q.OP_D, arith)
    got = cplx(fo.store())
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
    assert abs(g.plaquette() - 1.0) <= 1e-15
    for f in (g, fi, fo):
        f.close()


def _su3_field(orc, V, seed):
    rng = np.random.default_rng(seed)
    out = np.empty((V, 3, 3, 2))
    for v in range(V):
        m = rng.normal(size=(3, 3, 2))
        out[v] = orc.project_su3(m)
    return cplx(out)


@pytest.mark.parametrize("arith", [q.ARITH_F64, q.ARITH_DF64])
def test_gauge_covariance(gpu, orc, arith):
    L, th, kappa, mu = (4, 4, 2, 4), (np.pi, 0.0, 0.2, 0.0), 0.15, 0.03
    V = int(np.prod(L))
    U = cplx(orc.gauge_synthetic(L, 71, EPS_PLAQ_060))
    gx = _su3_field(orc, V, 72)
    c = coords(L)
    Ug = np.empty_like(U)
    for m in range(4):
        cn = c.copy()
        cn[:, m] = (cn[:, m] + 1) % L[m]
        fwd = cn[:, 0] + L[0] * (cn[:, 1] + L[1] * (cn[:, 2] + L[2] * cn[:, 3]))
        # U'_mu(x) = g(x) U_mu(x) g(x+mu)^+
        Ug[:, m] = gx @ U[:, m] @ np.conj(np.transpose(gx[fwd], (0, 2, 1)))
    psi = cplx(orc.gaussian_spinor(L, 73))
    psig = np.einsum("vab,vsb->vsa", gx, psi)
    g1, g2 = q.Gauge(L, th).load(real(U)), q.Gauge(L, th).load(real(Ug))
    f1, f2, o1, o2 = q.Field(L).load(real(psi)), q.Field(L).load(real(psig)), q.Field(L), q.Field(L)
    q.dslash(o1, f1, g1, kappa, mu, q.OP_D, arith)
    q.dslash(o2, f2, g2, kappa, mu, q.OP_D, arith)
    want = np.einsum("vab,vsb->vsa", gx, cplx(o1.store()))
    got = cplx(o2.store())
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
    assert abs(g1.plaquette() - g2.plaquette()) <= 1e-14
    for f in (g1, g2, f1, f2, o1, o2):
        f.close()


@pytest.mark.parametrize("L", [(8, 4, 4, 6), (48, 24, 24, 24)], ids=["small", "bench"])
def test_gamma5_hermiticity(gpu, L):
    """g5 D(mu) g5 = D(-mu)^+ as vectors (small) and as <chi, g5 D g5 psi> = <D(-mu) chi, psi> (bench size)."""
    th, kappa, mu = (np.pi, 0.0, 0.0, 0.0), 0.15, 0.04
    g = q.Gauge(L, th).synthetic(81, EPS_PLAQ_060)
    psi, chi = q.Field(L).gaussian(82), q.Field(L).gaussian(83)
    a, b = q.Field(L), q.Field(L)
    s = np.array([1, 1, -1, -1])[None, :, None, None]
    g5psi = q.Field(L).load(psi.store() * s)
    q.dslash(a, g5psi, g, kappa, mu, q.OP_D, q.ARITH_DF64)       # D(mu) g5 psi
    q.dslash(b, psi, g, kappa, -mu, q.OP_DDAG, q.ARITH_DF64)     # D(-mu)^+ psi
    lhs = a.store() * s
    if L[0] <= 8:
        rhs = b.store()
        assert np.max(np.abs(lhs - rhs)) <= 1e-13 * np.max(np.abs(rhs))
    c1 = np.vdot(cplx(chi.store()), cplx(lhs))
    c2 = chi.dot(b)
    assert abs(c1 - c2) <= 1e-12 * abs(c2)
    for f in (g, psi, chi, a, b, g5psi):
        f.close()


def test_bench_size_even_odd_solve_true_residual(gpu):
    """the 24^3 x 48 point-source solve converges on the FP64 true residual,
    recomputed here with the float-float operator"""
    L = (48, 24, 24, 24)
    g = q.Gauge(L, (np.pi, 0, 0, 0)).synthetic(1000, EPS_PLAQ_060)
    b, x, r = q.Field(L).point((0, 0, 0, 0), 0, 0), q.Field(L), q.Field(L)
    p = q.solve(x, b, g, 0.15, 0.0, solver=q.SOLVER_CGNR_EO, inner_prec=q.F16, tol=1e-10)
    assert p.status == 0 and p.true_residual <= 1e-10
    q.dslash(r, x, g, 0.15, 0.0, q.OP_D, q.ARITH_DF64)
    q.axpy(r, -1.0, b, r)  # r = Dx - b
    assert np.sqrt(r.norm2() / b.norm2()) <= 1e-10
    for f in (g, b, x, r):
        f.close()
