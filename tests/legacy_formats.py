"""The legacy propagator file formats in Python, for the file-format tests: a
restatement of the layouts lib/src/qcd_io.c reads and writes.

* CMI (qcd_io.c:907-982, 1685-1763): one vector, no header, big-endian
  float32 in the order [x][y][z][t][spin][colour][re, im].
* HMC (qcd_io.c:1200-1290): a text line "beta kappa mu L T" read with
  fscanf("%lf %lf %lf %d %d\\n"), then big-endian float64
  [column nu*3+c][x][y][z][t][spin][colour][re, im] for the 12 source
  columns.
* HMCV (qcd_io.c:1293-1383): the same header, then one vector.

fscanf's trailing "\\n" skips every whitespace byte after the header line,
so data whose first bytes are whitespace (0x09-0x0d, 0x20) start later than
the line's end; ``data_offset`` models that.
"""
import numpy as np


def _xyzt(v: np.ndarray, L) -> np.ndarray:
    """(V, 4, 3, 2) in qcd_lib site order (t fastest) -> [x][y][z][t][4][3][2]"""
    Lt, Lx, Ly, Lz = L
    return np.ascontiguousarray(v.reshape(Lz, Ly, Lx, Lt, 4, 3, 2).transpose(2, 1, 0, 3, 4, 5, 6))


def from_xyzt(a: np.ndarray, L) -> np.ndarray:
    Lt, Lx, Ly, Lz = L
    return np.ascontiguousarray(a.reshape(Lx, Ly, Lz, Lt, 4, 3, 2).transpose(2, 1, 0, 3, 4, 5, 6)).reshape(-1, 4, 3, 2)


def cmi_file(v, L) -> bytes:
    return _xyzt(v, L).astype(">f4").tobytes()


def header(L, beta=5.85, kappa=0.15, mu=0.004) -> bytes:
    return f"{beta:.6f} {kappa:.6f} {mu:.6f} {L[1]} {L[0]}\n".encode()


def hmc_file(cols, L, **kw) -> bytes:
    """cols: 12 vectors, column nu*3+c"""
    assert len(cols) == 12
    return header(L, **kw) + b"".join(_xyzt(c, L).astype(">f8").tobytes() for c in cols)


def hmcv_file(v, L, **kw) -> bytes:
    return header(L, **kw) + _xyzt(v, L).astype(">f8").tobytes()


WHITESPACE = b" \t\n\v\f\r"


def data_offset(blob: bytes) -> int:
    """where the reference's readers start the binary data of an HMC / HMCV
    file: after the header line and any whitespace bytes that follow it"""
    pos = blob.index(b"\n") + 1
    while pos < len(blob) and blob[pos] in WHITESPACE:
        pos += 1
    return pos


def read_vector(blob: bytes, L, col=0, hmc=True) -> np.ndarray:
    """the vector the reference's HMC (column col) or HMCV reader returns"""
    V = int(np.prod(L))
    off = data_offset(blob) + (col * 24 * V * 8 if hmc else 0)
    a = np.frombuffer(blob, dtype=">f8", count=24 * V, offset=off).astype(np.float64)
    return from_xyzt(a, L)
