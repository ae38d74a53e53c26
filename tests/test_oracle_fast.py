"""The timing build of the oracle (liboracle_fast.so: the 1D block products in
a vectorisable order, -ffast-math), which the CPU baseline and the reference
arm of bench.py time, computes the same apply as the checker build: same
topology and counts, coefficients within 1e-12 (CPU only)."""
import numpy as np

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, project


def test_fast_build_equals_checker():
    for order, basis in ((5, mw.INTERPOLATING), (7, mw.LEGENDRE)):
        mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
        P = mw.PoissonOperator(mra, 1e-3)
        f = project(mra, 1e-3, gaussian_sum(11, 3, (1.0, 30.0), (-3.0, 3.0)))
        a = oracle.Prepared(1e-3, mw.FunctionTree(mra), P, f).run(count_terms=True)
        b = oracle.Prepared(1e-3, mw.FunctionTree(mra), P, f).run(count_terms=True, fast=True)
        assert np.array_equal(a["idx"], b["idx"])
        assert a["node_terms"] == b["node_terms"] and a["components"] == b["components"]
        scale = np.abs(a["coefs"]).max()
        assert np.abs(a["coefs"] - b["coefs"]).max() <= 1e-12 * scale
