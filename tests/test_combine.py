"""Addition and multiplication (add.cpp, multiply.cpp): the CPU oracle against
closed forms -- integrals of a sum and of a product of Gaussians (a Gaussian)
(CPU; the GPU path is in test_gpu_combine.py)."""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import project

A0, B0 = np.array([0.3, 0.0, -0.2]), np.array([-0.1, 0.2, 0.1])


def inputs(basis, order, a1=0.8, a2=2.5):
    mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
    A = project(mra, 1e-7, [(1.0, a1, tuple(A0))])
    B = project(mra, 1e-7, [(1.0, a2, tuple(B0))])
    return mra, A, B


@pytest.mark.parametrize("basis,order", [(mw.INTERPOLATING, 5), (mw.LEGENDRE, 6)])
def test_oracle_sum_integral(basis, order):
    a1, a2 = 0.8, 2.5
    mra, A, B = inputs(basis, order, a1, a2)
    s = oracle.to_tree(oracle.combine(0, 1e-6, mw.FunctionTree(mra), [(2.0, A), (-1.5, B)]), mra)
    exact = 2.0 * (math.pi / a1) ** 1.5 - 1.5 * (math.pi / a2) ** 1.5
    assert s.integrate() == pytest.approx(exact, rel=1e-6)


@pytest.mark.parametrize("basis,order", [(mw.INTERPOLATING, 5), (mw.LEGENDRE, 6)])
def test_oracle_product_is_a_gaussian(basis, order):
    a1, a2 = 0.8, 2.5
    mra, A, B = inputs(basis, order, a1, a2)
    p = oracle.combine(1, 1e-6, mw.FunctionTree(mra), [(1.0, A), (1.0, B)])
    t = oracle.to_tree(p, mra)
    a = a1 + a2
    kfac = math.exp(-a1 * a2 / a * float(((A0 - B0) ** 2).sum()))
    assert t.integrate() == pytest.approx(kfac * (math.pi / a) ** 1.5, rel=1e-6)
    # squared norm of kfac exp(-a |r - P|^2): kfac^2 (pi / (2 a))^(3/2)
    assert p["square_norm"] == pytest.approx(kfac ** 2 * (math.pi / (2 * a)) ** 1.5, rel=1e-6)


def test_oracle_fixed_grid_sum_is_exact():
    # on a common fixed grid (max_iter = 0) the sum is the sum of the
    # coefficients: f + f = 2 f to the last bit
    mra, A, _ = inputs(mw.LEGENDRE, 5)
    g = mw.FunctionTree(mra)
    mw.copy_grid(g, A)
    s = oracle.combine(0, 1e-6, g, [(1.0, A), (1.0, A)], max_iter=0)
    x = A.export()
    key = {tuple(r): i for i, r in enumerate(s["idx"].tolist())}
    perm = [key[tuple(r)] for r in x["idx"].tolist()]
    np.testing.assert_array_equal(s["coefs"][perm], 2.0 * x["coefs"])
