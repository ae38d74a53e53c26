"""Fixed-grid applies (maxIter = 0 onto a fresh output grid) through the host
mirror's plan cache: the first apply of an (operator, output grid, input
topology) creates a level plan, the next ones replay it (stats["planned"] 2,
then 1).  The replayed level equals the level built by mwgpu_apply_level
(MWH_NO_PLAN_CACHE=1) -- FP64 to 1e-13, mixed within the mixed form's accuracy
of each other -- with the same node-term and component counts, and it follows
new input values (a rescaled input gives the rescaled output) and new input
objects of the same topology; a replay with an unchanged input uploads
nothing.
"""
import os

import numpy as np
import pytest

import mrcpp_gb300 as mw
from cases import gaussian_sum, project

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = project(mra, 1e-4, gaussian_sum(31, 4, (1.0, 100.0), (-5.0, 5.0)))
    grid = mw.FunctionTree(mra)
    mw.apply(1e-4, grid, P, f, precision=mw.FP64)
    return mra, P, f, grid


def fixed(mra, P, f, grid, form, cache=True):
    if not cache:
        os.environ["MWH_NO_PLAN_CACHE"] = "1"
    try:
        g = mw.FunctionTree(mra)
        mw.copy_grid(g, grid)
        st = mw.apply(1e-4, g, P, f, max_iter=0, precision=form)
    finally:
        os.environ.pop("MWH_NO_PLAN_CACHE", None)
    return g.export()["coefs"], st


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_replayed_plan_equals_built_level(gpu, case, form):
    mra, P, f, grid = case
    prec = mw.FP64 if form == "fp64" else mw.MIXED
    ref, sr = fixed(mra, P, f, grid, prec, cache=False)
    assert sr["planned"] == 0
    a, sa = fixed(mra, P, f, grid, prec)
    b, sb = fixed(mra, P, f, grid, prec)
    assert sa["planned"] in (1, 2) and sb["planned"] == 1
    # the replay moves no input bytes: the input is unchanged (and the plan
    # took over its resident device copy)
    assert sb["h2d_bytes"] == 0
    for s in (sa, sb):
        assert s["node_terms"] == sr["node_terms"] and s["components"] == sr["components"]
    rel = lambda x, y: np.linalg.norm(x - y) / np.linalg.norm(y)
    tol = 1e-13 if form == "fp64" else 2e-6
    assert rel(a, ref) <= tol and rel(b, ref) <= tol
    assert np.array_equal(a, b)


def test_plan_follows_new_input_values(gpu, case):
    mra, P, f, grid = case
    a, _ = fixed(mra, P, f, grid, mw.FP64)
    # new values of the same input tree (exact: scaling by 2)
    f.rescale(2.0)
    try:
        b, sb = fixed(mra, P, f, grid, mw.FP64)
    finally:
        f.rescale(0.5)
    assert sb["planned"] == 1
    assert np.linalg.norm(b - 2.0 * a) <= 1e-13 * np.linalg.norm(a)
    c, sc = fixed(mra, P, f, grid, mw.FP64)
    assert sc["planned"] == 1 and np.array_equal(c, a)
    # other input objects of one topology share a plan
    fx = f.export()
    h1, h2 = mw.FunctionTree(mra), mw.FunctionTree(mra)
    h1.load_flat(fx["idx"], fx["child0"], fx["coefs"])
    h2.load_flat(fx["idx"], fx["child0"], 3.0 * fx["coefs"])
    d1, s1 = fixed(mra, P, h1, grid, mw.FP64)
    d2, s2 = fixed(mra, P, h2, grid, mw.FP64)
    assert s1["planned"] in (1, 2) and s2["planned"] == 1
    assert np.linalg.norm(d1 - a) <= 1e-13 * np.linalg.norm(a)
    assert np.linalg.norm(d2 - 3.0 * a) <= 1e-13 * np.linalg.norm(a)


def test_batched_fixed_grids_replay_one_plan(gpu, case):
    # a batch of fixed-grid applies (one output grid per input) goes through
    # one cached plan for all pairs; each output equals the built level
    mra, P, _, _ = case
    fs = [project(mra, 1e-4, gaussian_sum(40 + i, n, (1.0, 100.0), (-5.0, 5.0))) for i, n in enumerate((1, 3, 2))]
    grids = []
    for f in fs:
        g = mw.FunctionTree(mra)
        mw.apply(1e-4, g, P, f, precision=mw.FP64)
        grids.append(g)

    def batch(form, cache=True):
        if not cache:
            os.environ["MWH_NO_PLAN_CACHE"] = "1"
        try:
            outs = []
            for g in grids:
                o = mw.FunctionTree(mra)
                mw.copy_grid(o, g)
                outs.append(o)
            st = mw.apply_batch(1e-4, outs, P, fs, max_iter=0, precision=form)
        finally:
            os.environ.pop("MWH_NO_PLAN_CACHE", None)
        return [o.export()["coefs"] for o in outs], st

    for form, tol in ((mw.FP64, 1e-13), (mw.MIXED, 2e-6)):
        ref, sr = batch(form, cache=False)
        a, sa = batch(form)
        b, sb = batch(form)
        assert sr["planned"] == 0 and sa["planned"] in (1, 2) and sb["planned"] == 1
        assert sb["h2d_bytes"] == 0
        for s in (sa, sb):
            assert s["node_terms"] == sr["node_terms"] and s["components"] == sr["components"]
        for x, y, r in zip(a, b, ref):
            assert np.linalg.norm(x - r) <= tol * np.linalg.norm(r)
            assert np.array_equal(x, y)
    # new values of one input: only that input goes up again
    fs[1].rescale(2.0)
    try:
        c, sc = batch(mw.FP64)
    finally:
        fs[1].rescale(0.5)
    assert sc["planned"] == 1 and 0 < sc["h2d_bytes"]
    ref64, _ = batch(mw.FP64, cache=False)
    assert np.linalg.norm(c[1] - 2.0 * ref64[1]) <= 1e-13 * np.linalg.norm(ref64[1])
    assert np.array_equal(c[0], ref64[0]) or np.linalg.norm(c[0] - ref64[0]) <= 1e-13 * np.linalg.norm(ref64[0])
