"""Hydrogen 1s fixed point of the Helmholtz operator: the reference's
known-answer test tests/operators/helmholtz_operator.cpp:131-198.

psi = exp(-r) / sqrt(pi), V = -1/r, E = -1/2, mu = sqrt(-2E) = 1; one
iteration psi' = -1/(2 pi) H[mu] (V psi) reproduces psi: |psi'| = 1 and
|psi' - psi| within the apply precision 3e-2.  World [-32, 32]^3 (scale -4,
2 x 2 x 2 boxes, scaling factor 2), interpolating order 5, operator built
from HelmholtzKernel(mu, 3e-3, r_min, r_max) as ConvolutionOperator(MRA,
kernel, 3e-3), functions projected at 3e-3.

CPU: the oracle's multiply, apply and add.  GPU: mrcpp_gb300's multiply, apply
(FP64 and mixed form) and add, also compared node by node with the oracle.
"""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle

PROJ_PREC, APPLY_PREC, BUILD_PREC = 3.0e-3, 3.0e-2, 3.0e-3


def psi_1s(r):
    # 2 Z^{3/2} exp(-Z rho / 2) Y_00 with rho = 2 Z |r|, Z = 1
    return 2.0 * np.exp(-np.linalg.norm(r, axis=1)) / math.sqrt(4.0 * math.pi)


def nuclear(r):
    return -1.0 / np.linalg.norm(r, axis=1)


def setup():
    mra = mw.MRA(order=5, basis=mw.INTERPOLATING, scale=-4, corner=(-1, -1, -1), nbox=(2, 2, 2), sf=2.0)
    mu = math.sqrt(-2.0 * -0.5)
    kernel = mw.helmholtz_kernel(mu, BUILD_PREC, mra.calcMinDistance(BUILD_PREC), mra.calcMaxDistance())
    H = mw.ConvolutionOperator(mra, kernel, BUILD_PREC)
    psi = mw.FunctionTree(mra)
    mw.project(PROJ_PREC, psi, psi_1s)
    V = mw.FunctionTree(mra)
    mw.project(PROJ_PREC, V, nuclear)
    return mra, H, psi, V


def grid_of(t):
    g = mw.FunctionTree(t.mra)
    mw.copy_grid(g, t)
    return g


def check_fixed_point(psi_np1, psi, diff_sq_norm):
    assert math.sqrt(psi.square_norm) == pytest.approx(1.0, rel=PROJ_PREC)
    assert math.sqrt(psi_np1.square_norm) == pytest.approx(1.0, rel=APPLY_PREC)
    assert math.sqrt(diff_sq_norm) < APPLY_PREC


def oracle_iteration(mra, H, psi, V):
    vpsi = oracle.to_tree(oracle.combine(1, -1.0, grid_of(psi), [(1.0, V), (1.0, psi)]), mra)
    psi_np1 = oracle.to_tree(oracle.apply(APPLY_PREC, grid_of(psi), H, vpsi, count_terms=False), mra)
    psi_np1.rescale(-1.0 / (2.0 * math.pi))
    d = oracle.combine(0, -1.0, grid_of(psi_np1), [(1.0, psi_np1), (-1.0, psi)])
    return vpsi, psi_np1, d


def test_projection_of_functions_and_kernel_operator():
    mra, H, psi, V = setup()
    # the 1s orbital is normalised and its projection integrates like exp(-r)/sqrt(pi)
    assert math.sqrt(psi.square_norm) == pytest.approx(1.0, rel=PROJ_PREC)
    assert psi.integrate() == pytest.approx(8.0 * math.sqrt(math.pi), rel=1e-4)
    x = np.array([[0.3, -0.2, 0.5]])
    # pointwise: prec bounds the L2 error relative to the norm
    assert psi.evalf(x[0]) == pytest.approx(psi_1s(x)[0], rel=1e-2)
    assert V.evalf(x[0]) == pytest.approx(nuclear(x)[0], rel=1e-2)
    assert H.size() == len(mw.helmholtz_kernel(1.0, BUILD_PREC, mra.calcMinDistance(BUILD_PREC), mra.calcMaxDistance())[0])
    # the callback's exception reaches the caller
    with pytest.raises(ZeroDivisionError):
        mw.project(PROJ_PREC, mw.FunctionTree(mra), lambda r: 1 / 0)


def test_oracle_hydrogen_fixed_point():
    mra, H, psi, V = setup()
    _, psi_np1, d = oracle_iteration(mra, H, psi, V)
    check_fixed_point(psi_np1, psi, d["square_norm"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [mw.FP64, mw.MIXED])
def test_gpu_hydrogen_fixed_point(gpu, precision):
    mra, H, psi, V = setup()
    vpsi = grid_of(psi)
    mw.multiply(-1.0, vpsi, 1.0, V, psi)
    psi_np1 = grid_of(psi)
    mw.apply(APPLY_PREC, psi_np1, H, vpsi, precision=precision)
    psi_np1.rescale(-1.0 / (2.0 * math.pi))
    d = grid_of(psi_np1)
    mw.add(-1.0, d, 1.0, psi_np1, -1.0, psi)
    check_fixed_point(psi_np1, psi, d.square_norm)

    # node by node against the oracle's iteration
    o_vpsi, o_psi_np1, _ = oracle_iteration(mra, H, psi, V)
    a, b = vpsi.export(), o_vpsi.export()
    assert np.array_equal(a["idx"], b["idx"])
    assert np.max(np.abs(a["coefs"] - b["coefs"])) <= 1e-12 * np.max(np.abs(b["coefs"]))
    a, b = psi_np1.export(), o_psi_np1.export()
    assert np.array_equal(a["idx"], b["idx"])
    tol = 1e-12 if precision == mw.FP64 else 1e-5
    assert np.linalg.norm(a["coefs"] - b["coefs"]) <= tol * np.linalg.norm(b["coefs"])
