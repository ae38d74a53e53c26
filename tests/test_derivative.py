"""Derivative operators (ABGVOperator, apply(out, D, inp, dir)): the CPU oracle
pinned to the reference's known-answer test, the operator's band structure,
and the output grid (CPU; the GPU path is in test_gpu_derivative.py)."""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import project


def reference_mra(order=5, basis=mw.INTERPOLATING):
    # tests/operators/derivative_operator.cpp:44-62: world scale -4, corner -1,
    # 2 boxes, scaling factor 2, interpolating k=5, max depth 20
    return mw.MRA(order=order, basis=basis, max_depth=20, scale=-4, corner=(-1, -1, -1), nbox=(2, 2, 2), sf=2.0)


def dgauss(r, r0, d):
    r = np.asarray(r) - np.asarray(r0)
    return -2.0 * r[..., d] * np.exp(-(r ** 2).sum(-1))


def point_error(tree, r0, d, n=400, seed=0):
    rng = np.random.default_rng(seed)
    pts = np.asarray(r0) + 0.8 * rng.normal(size=(n, 3))
    exact = dgauss(pts, r0, d)
    got = np.array([tree.evalf(p) for p in pts])
    return float(np.linalg.norm(got - exact) / np.linalg.norm(exact))


@pytest.mark.parametrize("a,b", [(0.5, 0.5), (0.0, 0.0)])
@pytest.mark.parametrize("d", [0, 1, 2])
def test_oracle_abgv_known_answer(a, b, d):
    # derivative_operator.cpp:85-124 (testDifferentiationABGV<3>): f = exp(-|r - r0|^2),
    # r0 = (pi, pi, pi), projected at prec / 10, prec = 1e-3; the derivative's
    # relative error is below prec (the reference measures it on the projected
    # derivative tree, here at sample points and through the exact norm
    # ||df||^2 = (pi / 2)^(3/2))
    prec = 1e-3
    mra = reference_mra()
    r0 = (math.pi, math.pi, math.pi)
    f = project(mra, prec / 10, [(1.0, 1.0, r0)])
    D = mw.ABGVOperator(mra, a, b)
    res = oracle.apply_derivative(mw.FunctionTree(mra), D, f, d)
    dg = oracle.to_tree(res, mra)
    assert point_error(dg, r0, d) < prec
    assert abs(res["square_norm"] - (math.pi / 2) ** 1.5) < prec * (math.pi / 2) ** 1.5


@pytest.mark.parametrize("basis", [mw.LEGENDRE, mw.INTERPOLATING])
def test_abgv_band_structure(basis):
    # ABGVCalculator.cpp:118-170: with a = b = 0 only l = 0 carries weight
    # (band 0); with a, b > 0 the neighbours l = -1, +1 do (band 1); every
    # depth l = -1..1 (BandWidthAdaptor refines the diagonal)
    mra = mw.MRA(box=(-32, 32), order=4, basis=basis)
    for (a, b), outer in (((0.0, 0.0), False), ((0.5, 0.5), True)):
        ex = mw.ABGVOperator(mra, a, b).export()
        assert list(ex["max_transl"]) == [1] * len(ex["max_transl"])
        nrm = ex["norms"].reshape(-1, 3, 4)  # per depth: l = -1, 0, 1
        assert (nrm[:, 1, 0] > 0).all() and (nrm[:, 1, 3] > 0).all()
        assert ((nrm[:, 0] > 0).any() and (nrm[:, 2] > 0).any()) == outer
        # scale doubling: the derivative at depth n + 1 is twice the one at n
        np.testing.assert_allclose(nrm[1:, 1, 0], 2.0 * nrm[:-1, 1, 0], rtol=1e-12)


def test_oracle_output_grid_is_widened_along_dir():
    # CopyAdaptor(inp, maxScale, bw) with bw[dir] = 1: the output grid holds
    # every node whose children, shifted by one box along dir, meet the input
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    f = project(mra, 1e-4, [(1.0, 3.0, (0.2, -0.1, 0.4))])
    fi = {tuple(r) for r in f.export()["idx"].tolist()}
    for a, grows in ((0.0, False), (0.5, True)):
        res = oracle.apply_derivative(mw.FunctionTree(mra), mw.ABGVOperator(mra, a, a), f, 0)
        gi = {tuple(r) for r in res["idx"].tolist()}
        assert fi <= gi
        assert (len(gi) > len(fi)) == grows
