"""LIME record helpers of the file-format tests (no GPU)."""
import numpy as np

from tests import lime_util


def test_record_layout_and_padding():
    r = lime_util.record("ildg-format", b"abc", True, False)
    assert len(r) == 144 + 8
    assert r[:4] == bytes.fromhex("456789ab") and r[4:6] == b"\0\x01" and r[6] == 0x80
    assert int.from_bytes(r[8:16], "big") == 3
    assert lime_util.parse(r) == [("ildg-format", True, False, b"abc")]


def test_ildg_payload_order():
    L = (2, 3, 2, 2)  # t, x, y, z
    V = 24
    u = np.arange(V * 72, dtype=np.float64).reshape(V, 4, 3, 3, 2)
    a = np.frombuffer(lime_util.ildg_payload(u, L), dtype=">f8").reshape(2, 2, 2, 3, 4, 3, 3, 2)
    # file (t=1, z=1, y=0, x=2, mu'=3 = t link) is site t + 2*(x + 3*(y + 2*z)), qcd_lib mu 0
    site = 1 + 2 * (2 + 3 * (0 + 2 * 1))
    assert np.array_equal(a[1, 1, 0, 2, 3], u[site, 0])
    assert np.array_equal(a[1, 1, 0, 2, 0], u[site, 1])
