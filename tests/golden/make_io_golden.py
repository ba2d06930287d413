"""Generate tests/golden/io_L4235.npz: files written by the reference's own
writers (lib/src/qcd_io.c compiled unmodified into oracle/_ref/libqcdio.so),
for the file-format tests on machines without the reference.

The LIME container those writers call is restated from the published LIME
format (oracle/lime_format.c; c-lime is not in the reference tree), so the
fixtures pin qcd_io.c's own part: record types, flags and XML text, payload
order, the direction remap and byte order. Inputs come from the oracle's
seeded generators. Run from the repository root where the reference tree
exists:

    python -c "import oracle.oracle as o; o.build()"
    python tests/golden/make_io_golden.py
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, ReferenceIO  # noqa: E402

EPS_PLAQ_060 = 0.43374
L = (4, 2, 3, 5)  # T, X, Y, Z: distinct extents catch index-order mistakes
MESSAGE = "written by qcd_writeGaugeLime"


def main():
    orc, rio = Oracle(), ReferenceIO()
    u = orc.gauge_synthetic(L, 71, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 72)
    rec = dict(L=np.array(L), u=u, v=v, message=np.frombuffer(MESSAGE.encode(), dtype=np.uint8))
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "f")
        assert rio.write_gauge(u, p, L, MESSAGE) == 0
        rec["conf_lime"] = np.fromfile(p, dtype=np.uint8)
        for key, t in (("prop_lime", ReferenceIO.PROP_LIME), ("source_lime", ReferenceIO.SOURCE_LIME),
                       ("vec_cmi", ReferenceIO.CMI)):
            assert rio.write_vector(v, p, L, t) == 0
            rec[key] = np.fromfile(p, dtype=np.uint8)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io_L4235.npz")
    np.savez(out, **rec)
    print("wrote", out)


if __name__ == "__main__":
    main()
