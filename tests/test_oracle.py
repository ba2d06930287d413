"""The CPU oracle pinned against the reference: committed golden vectors
(computed by the unmodified reference, see tests/golden/make_golden.py) and,
where the reference tree is present, the reference library itself."""
import numpy as np
import pytest

from oracle.oracle import site_rel_err

TOL = 1e-13  # per-site relative norm, the FP64 operator's parity bar


@pytest.mark.parametrize("case", ["wilson_L6442", "wilson_L4444_theta"])
def test_dslash_matches_golden(orc, golden, case):
    g = golden[case]
    L, th, kappa, tm = g["L"], g["theta"], float(g["kappa"]), float(g["tm"])
    m = 1.0 / (2.0 * kappa) - 4.0
    out = orc.dslash(g["v"], g["u"], L, th, m=m, tm=tm)
    for var in ("TMOp", "NoOptim", "NoScripts"):
        assert site_rel_err(out, g["out_" + var]) <= TOL
    q = orc.dslash(g["v"], g["u"], L, th, m=m, tm=tm, op="Q")
    assert site_rel_err(q, g["out_Q"]) <= TOL


@pytest.mark.parametrize("case", ["wilson_L6442", "wilson_L4444_theta"])
def test_blas_and_plaquette_match_golden(orc, golden, case):
    g = golden[case]
    v, w = g["v"], g["w"]
    assert abs(orc.norm(v) - float(g["norm_v"])) <= 1e-13 * float(g["norm_v"])
    d = orc.dot(v, w)
    ref = complex(*g["dot_vw"])
    assert abs(d - ref) <= 1e-12 * abs(ref) + 1e-12
    a = complex(*g["axpy_a"])
    assert np.array_equal(orc.axpy(a, v, w), g["axpy_vw"])  # same operation order: bit-exact
    assert abs(orc.plaquette(g["u"], g["L"]) - float(g["plaquette"])) <= 1e-14


@pytest.mark.parametrize("case", ["wilson_L6442", "wilson_L4444_theta"])
def test_gcr_shipped_matches_golden(orc, golden, case):
    g = golden[case]
    src = np.zeros_like(g["v"])
    src[0, 0, 0, 0] = 1.0
    sol, rc = orc.gcr(src, g["u"], g["L"], g["theta"], float(g["kappa"]), float(g["tm"]), 6, fixed=False)
    assert rc == 0
    assert np.max(np.abs(sol - g["gcr6_shipped"])) <= 1e-13 * np.max(np.abs(sol))


def test_golden_inputs_are_reproducible(orc, golden):
    # the generator that made the fixtures still produces them bit for bit
    from tests.golden.make_golden import CASES, EPS_PLAQ_060

    for name, c in CASES.items():
        g = golden[name]
        assert np.array_equal(orc.gauge_synthetic(c["L"], c["seed"], EPS_PLAQ_060), g["u"])
        assert np.array_equal(orc.gaussian_spinor(c["L"], c["seed"] + 100), g["v"])


# ------------------------------------------------------ against the reference
@pytest.mark.parametrize("L", [(4, 4, 4, 4), (8, 4, 2, 6), (2, 2, 2, 2)])
@pytest.mark.parametrize("tm", [0.0, -0.3])
def test_dslash_vs_reference(orc, ref, L, tm):
    th = (np.pi, 0.0, 0.5, 0.0)
    u = orc.gauge_synthetic(L, 3, 0.43374)
    v = orc.gaussian_spinor(L, 4)
    for var in ("TMOp", "NoOptim", "NoScripts"):
        assert site_rel_err(orc.dslash(v, u, L, th, kappa=0.14, tm=tm), ref.dslash(v, u, L, th, kappa=0.14, tm=tm, variant=var)) <= TOL
    assert site_rel_err(orc.dslash(v, u, L, th, kappa=0.14, tm=tm, op="Q"),
                        ref.dslash(v, u, L, th, kappa=0.14, tm=tm, variant="Q")) <= TOL


def test_dslash_non_su3_links_vs_reference(orc, ref):
    # arbitrary complex 3x3 links: the operator is linear in U, no SU(3) needed
    L = (4, 2, 4, 2)
    rng = np.random.default_rng(5)
    u = rng.normal(size=(np.prod(L), 4, 3, 3, 2))
    v = rng.normal(size=(np.prod(L), 4, 3, 2))
    th = (np.pi, 0, 0, 0)
    assert site_rel_err(orc.dslash(v, u, L, th, kappa=0.15), ref.dslash(v, u, L, th, kappa=0.15)) <= TOL


def test_setup_routines_vs_reference(orc, ref):
    L = (4, 4, 4, 4)
    u = orc.gauge_synthetic(L, 9, 0.43374)
    assert abs(orc.plaquette(u, L) - ref.plaquette(u, L)) <= 1e-14
    v = orc.gaussian_spinor(L, 10)
    assert np.max(np.abs(orc.gauss3d(v, u, L, 4.0, 1) - ref.gauss3d(v, u, L, 4.0, 1))) <= 1e-13
    # APE: the projection is computed by a different algorithm (Newton polar
    # iteration vs the reference's closed-form eigen-decomposition)
    assert np.max(np.abs(orc.ape3d(u, L, 0.5) - ref.ape3d(u, L, 0.5))) <= 1e-12
    rng = np.random.default_rng(2)
    M = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
    H = (M + M.conj().T) / 2
    H -= np.trace(H) / 3 * np.eye(3)
    Hf = np.stack([H.real, H.imag], -1)
    assert np.max(np.abs(orc.exp_iM(Hf) - ref.exp_iM(Hf))) <= 1e-14
    g = rng.normal(size=(3, 3, 2))
    assert np.max(np.abs(orc.project_su3(g) - ref.project_su3(g))) <= 1e-13


def test_gcr_vs_reference(orc, ref):
    L = (4, 4, 4, 4)
    th = (np.pi, 0, 0, 0)
    u = orc.gauge_synthetic(L, 1, 0.43374)
    src = orc.gaussian_spinor(L, 2)
    s_ref, rc1 = ref.gcr(src, u, L, th, 0.15, 0.02, 10)
    s_orc, rc2 = orc.gcr(src, u, L, th, 0.15, 0.02, 10, fixed=False)
    assert rc1 == rc2 == 0
    assert np.max(np.abs(s_ref - s_orc)) <= 1e-12 * np.max(np.abs(s_ref))


# --------------------------------------------------- oracle solver behaviour
def test_gcr_first_term_bug_stagnates(orc):
    """invert.c as shipped omits x = a00 c0 rho0; with it GCR converges."""
    L = (4, 4, 4, 4)
    th = (np.pi, 0, 0, 0)
    u = orc.gauge_synthetic(L, 1, 0.43374)
    src = np.zeros((256, 4, 3, 2))
    src[0, 0, 0, 0] = 1
    _, it_fixed, r_fixed = orc.invert_gcr(src, u, L, th, 0.15, 0.0, 16, fixed=True, maxres=1e-10, maxiter=200)
    _, it_shipped, r_shipped = orc.invert_gcr(src, u, L, th, 0.15, 0.0, 16, fixed=False, maxres=1e-10, maxiter=20)
    assert r_fixed <= 1e-10
    assert r_shipped > 1e-6


def test_oracle_solvers_true_residual(orc):
    L = (4, 4, 4, 4)
    th = (np.pi, 0, 0, 0)
    u = orc.gauge_synthetic(L, 1, 0.43374)
    b = orc.gaussian_spinor(L, 3)
    x, it, _ = orc.cgnr(b, u, L, th, 0.15, 0.0, tol=1e-12)
    assert orc.true_residual(x, b, u, L, th, 0.15) <= 1e-10
    # BiCGstab converges on a well-conditioned operator (small kappa)
    x, it, _ = orc.bicgstab(b, u, L, th, 0.11, 0.0, tol=1e-11)
    assert it > 0 and orc.true_residual(x, b, u, L, th, 0.11) <= 1e-10


def test_rng_counter_stream(orc):
    # fixed values: the GPU generator must reproduce these integers exactly
    bits = [orc.rng_bits(1, k) for k in range(4)]
    assert len(set(bits)) == 4
    z = orc.z4_spinor((2, 2, 2, 2), 7)
    vals = z[..., 0] + 1j * z[..., 1]
    assert set(np.unique(vals)).issubset({1, -1, 1j, -1j})
    counts = [np.sum(vals == c) for c in (1, -1, 1j, -1j)]
    assert min(counts) > 0.15 * vals.size


def test_twop_tables_match_reference(orc, ref):
    for mine, theirs in zip(orc.twop_tables(), ref.twop_tables()):
        assert np.array_equal(mine, theirs)


def test_twop_oracle_matches_reference_run(orc, ref):
    """twop.c itself (main() on in-memory inputs) against the restatement; the
    reference prints 7 significant digits (%+e), which bounds the agreement."""
    L, xsrc = (8, 4, 2, 4), (6, 3, 1, 2)
    V = int(np.prod(L))
    rng = np.random.default_rng(5)
    up, dn = rng.normal(size=(V, 4, 4, 3, 3, 2)), rng.normal(size=(V, 4, 4, 3, 3, 2))
    u = orc.gauge_synthetic(L, 6, 0.43374)
    moms = [(0, 0, 0), (1, 1, 0), (-1, 0, 2)]
    c_ref = ref.twop(u, up, dn, L, xsrc, 0, 7, moms)
    c_orc = orc.twop_proton(up, dn, L, xsrc, 0, 7, moms)
    assert np.max(np.abs(c_orc - c_ref)) <= 2e-6 * np.max(np.abs(c_ref))


@pytest.mark.parametrize("case", ["twop_L8442", "twop_L8442_smeared"])
def test_twop_oracle_matches_golden(orc, golden, case):
    from tests.golden.make_golden import TWOP_MOMS, twop_inputs

    g = golden[case]
    L = tuple(int(x) for x in g["L"])
    u, cu, cd, prop = twop_inputs(orc, L, int(g["seed"]))
    if int(g["nsmear"]):
        ua = u
        for _ in range(int(g["nape"])):
            ua = orc.ape3d(ua, L, 0.5)
        for cols in (cu, cd):
            for k in range(12):
                for _ in range(int(g["nsmear"])):
                    for t in range(L[0]):
                        cols[k] = orc.gauss3d(cols[k], ua, L, 4.0, t)
    corr = orc.twop_proton(prop(cu), prop(cd), L, tuple(int(x) for x in g["xsrc"]), int(g["t0"]), int(g["t1"]),
                           TWOP_MOMS)
    assert np.max(np.abs(corr - g["corr"])) <= 2e-6 * np.max(np.abs(g["corr"]))


@pytest.mark.parametrize("case", ["wilson_L6442", "wilson_L4444_theta"])
def test_timed_cpu_operator_matches_golden(orc, golden, case):
    """the CPU baseline's timed operator (half-spinor algorithm, -O3) computes
    the reference's D: golden outputs of qcd_applyWilsonTMOp at 1e-13 per site"""
    g = golden[case]
    L, th, kappa, tm = g["L"], g["theta"], float(g["kappa"]), float(g["tm"])
    out = orc.dslash_fast(g["v"], g["u"], L, th, m=1.0 / (2.0 * kappa) - 4.0, tm=tm)
    assert site_rel_err(out, g["out_TMOp"]) <= TOL


def test_timed_cpu_operator_vs_checker_all_phases(orc):
    L, th = (6, 4, 2, 4), (np.pi, 0.4, -0.3, 1.1)
    u = orc.gauge_synthetic(L, 9, 0.43374)
    v = orc.gaussian_spinor(L, 10)
    for tm in (0.0, 0.21):
        assert site_rel_err(orc.dslash_fast(v, u, L, th, kappa=0.14, tm=tm),
                            orc.dslash(v, u, L, th, kappa=0.14, tm=tm)) <= TOL


def test_timed_cpu_operator_runs_at_the_reference_speed(orc, ref):
    """the CPU baseline times the reference's algorithm, not a slower one: on
    the benchmark's 24^3 x 48 lattice, on this core, its apply takes within
    15% of the reference's own qcd_applyWilsonTMOp. Each round takes the best
    of ten applies of each, interleaved; a host shared with other processes
    (or still busy with a build) can slow a whole round, so up to six rounds
    are measured and one within the bound suffices."""
    import time

    L, th = (48, 24, 24, 24), (np.pi, 0.0, 0.0, 0.0)
    u = orc.gauge_synthetic(L, 1000, 0.43374)
    v = orc.gaussian_spinor(L, 2000)
    out = np.empty_like(v)
    r = ref.dslash(v, u, L, th, kappa=0.15)
    orc.dslash_fast(v, u, L, th, kappa=0.15, out=out)
    assert site_rel_err(out, r) <= TOL
    ratios = []
    for _ in range(6):
        t_fast, t_ref = [], []
        for _ in range(10):
            t0 = time.perf_counter()
            orc.dslash_fast(v, u, L, th, kappa=0.15, out=out)
            t_fast.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            ref.dslash(v, u, L, th, kappa=0.15)
            t_ref.append(time.perf_counter() - t0)
        ratios.append(min(t_fast) / min(t_ref))
        if 0.85 <= ratios[-1] <= 1.15:
            break
    assert 0.85 <= ratios[-1] <= 1.15, ratios
