"""Writes tests/golden/mwfilters_ref.npz and tests/golden/deriv_tables_ref.npz
from the reference's shipped filter tables (share/mwfilters of
MRChemSoft/mrcpp), for the orders the tests compare.

Run with the path of a checkout of the reference as its one argument:
    python tests/golden/make_golden.py <mrcpp checkout>
The first fixture holds H0 and G0 (K x K, row-major as stored) and the
left/right cross-correlation matrices (K^2 x 2K) for Legendre (L) and
Interpolating (I); the second the derivative tables of the PH and B-spline
derivative operators ([S_+1; S_0; S_-1], 3K x K as stored in the text files
PHCalculator.cpp:44-74 and BSCalculator.cpp:44-74 read), key
"<L|I>_<ph|bs><derivative order>_<k>".
"""
import os
import sys

import numpy as np

ORDERS_FILTER = [0, 1, 2, 3, 5, 7, 9, 11, 15, 19]
ORDERS_CC = [1, 3, 5, 7, 9]
ORDERS_DERIV = [1, 5, 7, 9]
DERIV_FILES = {"ph": ("%s_ph_deriv_%d.txt", (1, 2)), "bs": ("%s_b-spline-deriv%d.txt", (1, 2, 3))}


def read_deriv_file(path, kp1_max):
    """{kp1: (3 kp1 x kp1) array} of one derivative table file: for kp1 = 2, 3, ...
    a line holding kp1, then 3 kp1 lines of kp1 numbers."""
    out = {}
    with open(path) as fh:
        lines = fh.read().split("\n")
    pos = 0
    for kp1 in range(2, kp1_max):
        if int(lines[pos].split()[0]) != kp1:
            raise ValueError("%s: orders do not match at kp1 = %d" % (path, kp1))
        rows = [[float(x) for x in lines[pos + 1 + i].split()] for i in range(3 * kp1)]
        out[kp1] = np.array(rows)
        pos += 1 + 3 * kp1
    return out


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
    der = {}
    for t in "LI":
        for kind, (pattern, orders) in DERIV_FILES.items():
            for n in orders:
                tabs = read_deriv_file(os.path.join(d, pattern % (t, n)), 21)
                for k in ORDERS_DERIV:
                    der["%s_%s%d_%d" % (t, kind, n, k)] = tabs[k + 1]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "deriv_tables_ref.npz")
    np.savez_compressed(path, **der)
    print("wrote", path, len(der), "arrays")


if __name__ == "__main__":
    main()
