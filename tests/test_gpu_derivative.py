"""GPU parity of the derivative path (apply(out, ABGVOperator, inp, dir),
mwgpu_apply_derivative through the C-ABI) against the CPU oracle: identical
output grid and (g, f) counts, FP64 coefficients within 1e-12 of the largest."""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, project, rel_errors

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


@pytest.mark.parametrize("basis,order", [(mw.INTERPOLATING, 5), (mw.LEGENDRE, 7)])
@pytest.mark.parametrize("a,b", [(0.5, 0.5), (0.0, 0.0), (1.0, 0.0)])
def test_abgv_gpu_vs_oracle(gpu, basis, order, a, b):
    mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
    f = project(mra, 1e-4, gaussian_sum(17, 3, (1.0, 30.0), (-2.0, 2.0)))
    D = mw.ABGVOperator(mra, a, b)
    for d in range(3):
        g = mw.FunctionTree(mra)
        st = mw.apply(g, D, f, d)
        ref = oracle.apply_derivative(mw.FunctionTree(mra), D, f, d)
        gx = g.export()
        same, perm = match(gx, ref)
        assert same, "output grid differs from the oracle"
        mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
        assert mx <= FP64_TOL and l2 <= FP64_TOL, (mx, l2)
        assert st["node_terms"] == ref["node_terms"]
        assert st["components"] == ref["components"]
        assert g.square_norm == pytest.approx(ref["square_norm"], rel=1e-12)


def test_abgv_gpu_known_answer(gpu):
    # the reference's setting (derivative_operator.cpp:85-124) on the GPU path
    prec = 1e-3
    mra = mw.MRA(order=5, basis=mw.INTERPOLATING, max_depth=20, scale=-4, corner=(-1, -1, -1), nbox=(2, 2, 2), sf=2.0)
    r0 = (math.pi, math.pi, math.pi)
    f = project(mra, prec / 10, [(1.0, 1.0, r0)])
    g = mw.FunctionTree(mra)
    mw.apply(g, mw.ABGVOperator(mra, 0.5, 0.5), f, 0)
    rng = np.random.default_rng(1)
    pts = np.asarray(r0) + 0.8 * rng.normal(size=(400, 3))
    exact = -2.0 * (pts[:, 0] - r0[0]) * np.exp(-((pts - np.asarray(r0)) ** 2).sum(-1))
    got = np.array([g.evalf(p) for p in pts])
    assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < prec
    assert abs(g.square_norm - (math.pi / 2) ** 1.5) < prec * (math.pi / 2) ** 1.5


def test_derivative_after_mixed_apply(gpu):
    # the derivative is FP64 whatever precision mode the last apply left, and
    # a GenNode pool made in the mixed form does not leak into it
    mra = mw.MRA(box=(-20, 20), order=7, basis=mw.LEGENDRE)
    f = project(mra, 1e-4, gaussian_sum(23, 2, (2.0, 20.0), (-1.0, 1.0)))
    P = mw.PoissonOperator(mra, 1e-4)
    mw.apply(1e-4, mw.FunctionTree(mra), P, f, precision=mw.MIXED)
    D = mw.ABGVOperator(mra, 0.5, 0.5)
    g = mw.FunctionTree(mra)
    mw.apply(g, D, f, 2)
    ref = oracle.apply_derivative(mw.FunctionTree(mra), D, f, 2)
    same, perm = match(g.export(), ref)
    assert same
    mx, _ = rel_errors(g.export()["coefs"], ref["coefs"][perm])
    assert mx <= FP64_TOL
