"""Input trees stay on the device between applies (the host tree owns its
device copy, reused while the tree is unchanged): a repeated apply moves no
input bytes and gives the same result; every change of the host tree
(rescale, projection, import) makes the next apply upload it again, and the
result follows the change (linearity for the rescale).  The copy serves both
forms in turn.
"""
import numpy as np
import pytest

import mrcpp_gb300 as mw
from cases import gaussian_sum, project

pytestmark = pytest.mark.gpu


def tree_bytes(f):
    x = f.export()
    return x["coefs"].nbytes


def fixed_apply(prec, grid, P, f, form):
    g = mw.FunctionTree(grid.mra)
    mw.copy_grid(g, grid)
    st = mw.apply(prec, g, P, f, max_iter=0, precision=form)
    return g.export()["coefs"], st


def test_repeated_apply_reuses_the_input(gpu):
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = project(mra, 1e-4, gaussian_sum(5, 4, (1.0, 50.0), (-4.0, 4.0)))
    grid = mw.FunctionTree(mra)
    mw.apply(1e-4, grid, P, f, precision=mw.FP64)
    nb = tree_bytes(f)
    a, st_a = fixed_apply(1e-4, grid, P, f, mw.MIXED)
    b, st_b = fixed_apply(1e-4, grid, P, f, mw.MIXED)
    # the apply that made the grid uploaded f: these upload only the output
    # topology and the level lists
    assert st_a["h2d_bytes"] < nb / 10 and st_b["h2d_bytes"] < nb / 10
    assert np.array_equal(a, b)
    # the other form on the same device copy, then back
    c64, _ = fixed_apply(1e-4, grid, P, f, mw.FP64)
    d, _ = fixed_apply(1e-4, grid, P, f, mw.MIXED)
    assert np.array_equal(a, d)
    assert np.abs(c64 - a).max() <= 1e-5 * np.abs(c64).max()
    # a changed input is uploaded again and the result follows it
    f.rescale(2.0)
    e, st_e = fixed_apply(1e-4, grid, P, f, mw.FP64)
    assert st_e["h2d_bytes"] >= nb
    np.testing.assert_allclose(e, 2.0 * c64, rtol=0, atol=1e-12 * np.abs(c64).max())
    # a new projection into the same tree object
    mw.project(1e-4, f, gaussian_sum(6, 3, (1.0, 50.0), (-4.0, 4.0)))
    h, _ = fixed_apply(1e-4, grid, P, f, mw.FP64)
    fresh = mw.FunctionTree(mra)
    x = f.export()
    fresh.load_flat(x["idx"], x["child0"], x["coefs"])
    k, st_k = fixed_apply(1e-4, grid, P, fresh, mw.FP64)
    assert st_k["h2d_bytes"] >= tree_bytes(fresh)
    assert np.array_equal(h, k)


def test_batch_reuses_inputs(gpu):
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    fs = [project(mra, 1e-4, gaussian_sum(100 + i, 2 + i, (1.0, 50.0), (-4.0, 4.0))) for i in range(4)]
    nb = sum(tree_bytes(f) for f in fs)
    runs = []
    for _ in range(2):
        outs = [mw.FunctionTree(mra) for _ in fs]
        st = mw.apply_batch(1e-4, outs, P, fs, precision=mw.MIXED)
        runs.append(([o.export()["coefs"] for o in outs], st))
    assert runs[1][1]["h2d_bytes"] < nb / 10
    for a, b in zip(runs[0][0], runs[1][0]):
        assert np.array_equal(a, b)
