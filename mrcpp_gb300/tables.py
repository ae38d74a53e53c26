"""Reader of mrcpp_gb300/data/mwtables.bin (written by data/gen_mwtables.py).

Kinds: 0 = H0, 1 = G0 (K x K, row i = parent function i), 2 = cross-correlation
left, 3 = right (K^2 x 2K).  Types: 0 = Legendre, 1 = Interpolating.
"""
import os
import struct

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "mwtables.bin")
H0, G0, CLEFT, CRIGHT = 0, 1, 2, 3


def load(path=PATH):
    with open(path, "rb") as fh:
        d = fh.read()
    if d[:4] != b"MWTB":
        raise ValueError("not an MW table file: %s" % path)
    _, n = struct.unpack("<ii", d[4:12])
    off = 12
    out = {}
    for _ in range(n):
        kind, typ, k, r, c = struct.unpack("<iiiii", d[off:off + 20])
        off += 20
        out[(kind, typ, k)] = np.frombuffer(d[off:off + 8 * r * c], dtype="<f8").reshape(r, c).copy()
        off += 8 * r * c
    return out
