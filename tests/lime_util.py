"""LIME records in Python for the file-format tests: a restatement of the
LIME v1 record layout (magic 0x456789ab, version, MB/ME flags, data length,
128-byte type, data padded to 8 bytes) and of qcd_lib's ILDG / ETMC data
order (lib/src/qcd_io.c:204-399, 984-1150)."""
import struct

import numpy as np

MAGIC = 0x456789AB


def record(rtype: str, data: bytes, mb: bool, me: bool) -> bytes:
    flags = (0x80 if mb else 0) | (0x40 if me else 0)
    head = struct.pack(">IHBBQ", MAGIC, 1, flags, 0, len(data)) + rtype.encode().ljust(128, b"\0")
    return head + data + b"\0" * ((-len(data)) % 8)


def parse(blob: bytes):
    """[(type, mb, me, data)]"""
    out, pos = [], 0
    while pos < len(blob):
        magic, ver, flags, _, n = struct.unpack(">IHBBQ", blob[pos:pos + 16])
        assert magic == MAGIC and ver == 1
        rtype = blob[pos + 16:pos + 144].split(b"\0")[0].decode()
        data = blob[pos + 144:pos + 144 + n]
        out.append((rtype, bool(flags & 0x80), bool(flags & 0x40), data))
        pos += 144 + n + (-n) % 8
    return out


def ildg_payload(u: np.ndarray, L, prec=64) -> bytes:
    """u: (V, 4, 3, 3, 2) in qcd_lib order (site t fastest, mu = t,x,y,z) ->
    big-endian [t][z][y][x][mu'][3][3][2] with mu' = x,y,z,t."""
    Lt, Lx, Ly, Lz = L
    a = u.reshape(Lz, Ly, Lx, Lt, 4, 3, 3, 2)              # site index t + Lt*(x + Lx*(y + Ly*z))
    a = a.transpose(3, 0, 1, 2, 4, 5, 6, 7)                # [t][z][y][x][mu]...
    a = a[:, :, :, :, [1, 2, 3, 0]]                          # file mu' = 0..3 -> qcd_lib mu = (mu'+1)%4
    return np.ascontiguousarray(a).astype(">f8" if prec == 64 else ">f4").tobytes()


def etmc_payload(v: np.ndarray, L, prec=64) -> bytes:
    Lt, Lx, Ly, Lz = L
    a = v.reshape(Lz, Ly, Lx, Lt, 4, 3, 2).transpose(3, 0, 1, 2, 4, 5, 6)
    return np.ascontiguousarray(a).astype(">f8" if prec == 64 else ">f4").tobytes()


def etmc_array(data: bytes, L, prec=64) -> np.ndarray:
    """ETMC payload -> (V, 4, 3, 2) in qcd_lib order (the inverse of etmc_payload)"""
    Lt, Lx, Ly, Lz = L
    a = np.frombuffer(data, dtype=">f8" if prec == 64 else ">f4").astype(np.float64)
    return np.ascontiguousarray(a.reshape(Lt, Lz, Ly, Lx, 4, 3, 2).transpose(1, 2, 3, 0, 4, 5, 6)).reshape(-1, 4, 3, 2)


def ildg_file(u, L, prec=64) -> bytes:
    xml = (f"<?xml version=\"1.0\"?>\n<ildgFormat>\n<field>su3gauge</field>\n<precision>{prec}</precision>\n"
           f"<lx>{L[1]}</lx><ly>{L[2]}</ly><lz>{L[3]}</lz><lt>{L[0]}</lt>\n</ildgFormat>").encode()
    return (record("ildg-format", xml, True, False) + record("xlf-info", b"test", False, False) +
            record("ildg-binary-data", ildg_payload(u, L, prec), False, True))


def etmc_file(v, L, prec=64) -> bytes:
    xml = (f"<?xml version=\"1.0\"?>\n<etmcFormat>\n<field>diracFermion</field>\n<precision>{prec}</precision>\n"
           f"<lx>{L[1]}</lx><ly>{L[2]}</ly><lz>{L[3]}</lz><lt>{L[0]}</lt>\n</etmcFormat>").encode()
    return (record("propagator-type", b"DiracFermion_Sink", True, True) +
            record("etmc-propagator-format", xml, True, True) +
            record("scidac-binary-data", etmc_payload(v, L, prec), True, True))
