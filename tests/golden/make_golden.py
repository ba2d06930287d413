"""Generate the golden vectors under tests/golden from the reference itself.

Inputs come from the oracle's seeded generators; every output is computed by
the reference library compiled unmodified (oracle/_ref/libqcdref.so), so the
fixtures pin the reference's own behaviour, independently of this project's
restatement. Run from the repository root where the reference tree exists:

    python -c "import oracle.oracle as o; o.build()"
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, Reference  # noqa: E402

EPS_PLAQ_060 = 0.43374  # synthetic links with mean plaquette ~0.60

CASES = {
    # distinct extents catch index-order mistakes; antiperiodic in t
    "wilson_L6442": dict(L=(6, 4, 4, 2), theta=(np.pi, 0.0, 0.0, 0.0), kappa=0.15, tm=0.1, seed=11),
    # boundary phases in every direction, non-zero twisted mass
    "wilson_L4444_theta": dict(L=(4, 4, 4, 4), theta=(np.pi, 0.3, -0.7, 1.1), kappa=0.13, tm=0.05, seed=12),
}


def main():
    orc, ref = Oracle(), Reference()
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for name, c in CASES.items():
        L, th, kappa, tm = c["L"], c["theta"], c["kappa"], c["tm"]
        u = orc.gauge_synthetic(L, c["seed"], EPS_PLAQ_060)
        v = orc.gaussian_spinor(L, c["seed"] + 100)
        w = orc.gaussian_spinor(L, c["seed"] + 200)
        m = 1.0 / (2.0 * kappa) - 4.0
        rec = dict(L=np.array(L), theta=np.array(th), kappa=kappa, tm=tm, u=u, v=v, w=w)
        for var in ("TMOp", "NoOptim", "NoScripts", "Q"):
            rec["out_" + var] = ref.dslash(v, u, L, th, m=m, tm=tm, variant=var)
        rec["plaquette"] = ref.plaquette(u, L)
        rec["norm_v"] = ref.blas(0, np.zeros_like(v), v, v, L=L)[0]
        rec["dot_vw"] = ref.blas(1, np.zeros_like(v), v, w, L=L)
        a = 0.3 - 1.7j
        o = np.zeros_like(v)
        ref.blas(2, o, v, w, a, L=L)
        rec["axpy_vw"] = o
        rec["axpy_a"] = np.array([a.real, a.imag])
        src = np.zeros_like(v)
        src[0, 0, 0, 0] = 1.0
        sol, rc = ref.gcr(src, u, L, th, kappa, tm, 6)
        assert rc == 0
        rec["gcr6_shipped"] = sol
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **rec)
        print("wrote", name)


# proton two-point function (twop.c run on in-memory inputs): propagator
# column k of up / down = oracle Gaussian spinor of seed TWOP_SEED + k / + 100 + k
TWOP = {
    "twop_L8442": dict(L=(8, 4, 4, 2), xsrc=(3, 1, 2, 0), t0=0, t1=7, nsmear=0, nape=0, seed=21),
    "twop_L8442_smeared": dict(L=(8, 4, 4, 2), xsrc=(5, 0, 3, 1), t0=1, t1=6, nsmear=2, nape=1, seed=22),
}
TWOP_MOMS = [(0, 0, 0), (1, 0, 0), (0, -1, 1), (2, 1, 0)]


def twop_inputs(orc, L, seed):
    u = orc.gauge_synthetic(L, seed, EPS_PLAQ_060)
    V = int(np.prod(L))
    cols = lambda off: [orc.gaussian_spinor(L, 1000 * seed + off + k) for k in range(12)]  # noqa: E731
    # D[v][mu][nu][c1][c2]: column k = nu * 3 + c2 holds [v][mu][c1]
    prop = lambda cs: np.stack(cs, axis=0).reshape(4, 3, V, 4, 3, 2).transpose(2, 3, 0, 4, 1, 5)  # noqa: E731
    return u, cols(0), cols(100), prop


def main_twop():
    orc, ref = Oracle(), Reference()
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for name, c in TWOP.items():
        L = c["L"]
        u, cu, cd, prop = twop_inputs(orc, L, c["seed"])
        corr = ref.twop(u, np.ascontiguousarray(prop(cu)), np.ascontiguousarray(prop(cd)), L, c["xsrc"], c["t0"],
                        c["t1"], TWOP_MOMS, nsmear=c["nsmear"], alpha=4.0, nape=c["nape"], alpha_ape=0.5)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), corr=corr, moms=np.array(TWOP_MOMS),
                            **{k: np.array(v) for k, v in c.items()})
        print("wrote", name)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "twop":
        main_twop()
        sys.exit(0)
    main()
