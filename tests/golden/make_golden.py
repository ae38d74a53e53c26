"""Writes tests/golden/mwfilters_ref.npz from the reference's shipped filter
tables (share/mwfilters of MRChemSoft/mrcpp), for the orders the tests compare.

Run with the path of a checkout of the reference as its one argument:
    python tests/golden/make_golden.py <mrcpp checkout>
The fixture holds H0 and G0 (K x K, row-major as stored) and the left/right
cross-correlation matrices (K^2 x 2K) for Legendre (L) and Interpolating (I).
"""
import os
import sys

import numpy as np

ORDERS_FILTER = [0, 1, 2, 3, 5, 7, 9, 11, 15, 19]
ORDERS_CC = [1, 3, 5, 7, 9]


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of an mrcpp checkout>")
    ref = sys.argv[1]
    d = os.path.join(ref, "share", "mwfilters")
    out = {}
    for t in "LI":
        for k in ORDERS_FILTER:
            K = k + 1
            out["%s_H0_%d" % (t, k)] = np.fromfile(os.path.join(d, "%s_H0_%d" % (t, k))).reshape(K, K)
            out["%s_G0_%d" % (t, k)] = np.fromfile(os.path.join(d, "%s_G0_%d" % (t, k))).reshape(K, K)
        for k in ORDERS_CC:
            K = k + 1
            for side in ("left", "right"):
                out["%s_c_%s_%d" % (t, side, k)] = np.fromfile(os.path.join(d, "%s_c_%s_%d" % (t, side, k))).reshape(K * K, 2 * K)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mwfilters_ref.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "arrays")


if __name__ == "__main__":
    main()
