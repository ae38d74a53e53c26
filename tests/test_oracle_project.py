"""The oracle's projection (project.cpp:41-66, ProjectionCalculator.cpp:34-51;
quadrature and value-to-coefficient maps computed with numpy) against the
host mirror's (mw_project.cpp), on the CPU: the same grid and coefficients
within 1e-13 of the largest, for a Slater function and a Gaussian sum in both
bases."""
import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, rel_errors


def slater(r):
    return np.exp(-np.linalg.norm(r, axis=1)) / np.sqrt(np.pi)


def gsum(gs):
    def f(r):
        v = np.zeros(len(r))
        for c, a, R in gs:
            v += c * np.exp(-a * ((r - np.asarray(R)) ** 2).sum(axis=1))
        return v
    return f


@pytest.mark.parametrize("basis,order", [(mw.LEGENDRE, 7), (mw.INTERPOLATING, 5)])
@pytest.mark.parametrize("which", ["slater", "gaussians"])
def test_oracle_projection_equals_host(basis, order, which):
    mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
    f = slater if which == "slater" else gsum(gaussian_sum(31, 3, (1.0, 40.0), (-2.0, 2.0)))
    ref = oracle.project(1e-5, mw.FunctionTree(mra), f)
    t = mw.FunctionTree(mra)
    mw.project(1e-5, t, f)
    tx = t.export()
    same, perm = match(tx, ref)
    assert same
    mx, l2 = rel_errors(tx["coefs"], ref["coefs"][perm])
    assert mx <= 1e-13 and l2 <= 1e-13, (mx, l2)
    if which == "slater":
        assert ref["square_norm"] == pytest.approx(1.0, abs=1e-6)
