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


# PHOperator / BSOperator (src/operators/PHOperator.cpp, BSOperator.cpp) from
# the reference's tables (tests/golden/deriv_tables_ref.npz, written into a
# filter directory in the reference's file format)
def _table_operator(tmp_path, mra, kind, n, t, k):
    from test_deriv_tables import filter_dir

    d = filter_dir(tmp_path, t, kind, n, k)
    return (mw.PHOperator if kind == "ph" else mw.BSOperator)(mra, n, d)


@pytest.mark.parametrize("kind,n", [("ph", 1), ("ph", 2), ("bs", 1), ("bs", 2), ("bs", 3)])
@pytest.mark.parametrize("basis,t,k", [(mw.LEGENDRE, "L", 7), (mw.INTERPOLATING, "I", 5)])
def test_table_derivatives_gpu_vs_oracle(gpu, tmp_path, kind, n, basis, t, k):
    mra = mw.MRA(box=(-20, 20), order=k, basis=basis)
    f = project(mra, 1e-4, gaussian_sum(17, 3, (1.0, 30.0), (-2.0, 2.0)))
    D = _table_operator(tmp_path, mra, kind, n, t, k)
    for d in (0, 2):
        g = mw.FunctionTree(mra)
        st = mw.apply(g, D, f, d)
        ref = oracle.apply_derivative(mw.FunctionTree(mra), D, f, d)
        gx = g.export()
        same, perm = match(gx, ref)
        assert same, "output grid differs from the oracle"
        mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
        assert mx <= FP64_TOL and l2 <= FP64_TOL, (kind, n, d, mx, l2)
        assert st["node_terms"] == ref["node_terms"] and st["components"] == ref["components"]


@pytest.mark.parametrize("n,tol", [(1, 1e-4), (2, 1e-3), (3, 1e-2)])
def test_bspline_derivative_known_answer(gpu, tmp_path, n, tol):
    # d^n/dx^n of exp(-r^2) (the B-spline derivative is the one for smooth functions)
    mra = mw.MRA(box=(-20, 20), order=7, basis=mw.LEGENDRE)
    f = project(mra, 1e-6, [(1.0, 1.0, (0.0, 0.0, 0.0))])
    D = _table_operator(tmp_path, mra, "bs", n, "L", 7)
    g = mw.FunctionTree(mra)
    mw.apply(g, D, f, 0)
    rng = np.random.default_rng(3)
    pts = 0.8 * rng.normal(size=(300, 3))
    x, e = pts[:, 0], np.exp(-(pts ** 2).sum(-1))
    exact = {1: -2.0 * x * e, 2: (4.0 * x * x - 2.0) * e, 3: (-8.0 * x ** 3 + 12.0 * x) * e}[n]
    got = np.array([g.evalf(p) for p in pts])
    assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < tol
