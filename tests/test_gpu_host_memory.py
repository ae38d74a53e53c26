"""Tree coefficients of 4 MiB and more live in page-locked host memory, so
the input upload and result download of an apply run as DMA: on a GPU host the
blocks are page-locked, freed blocks wait in the cache and are taken again by
the next tree of that size, and an apply whose input is uploaded again from
page-locked memory (the tree marked changed) gives the same coefficients as the
first apply of it and as the oracle.
"""
import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, project, rel_errors

pytestmark = pytest.mark.gpu


def test_page_locked_trees(gpu):
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    prec = 1e-4
    f = project(mra, prec, gaussian_sum(2026, 6, (1.0, 100.0), (-5.0, 5.0)))
    nbytes = f.export()["coefs"].nbytes
    assert nbytes >= 4 << 20
    st = mw.pinned_stats()
    assert st["state"] == 1 and st["live_bytes"] >= nbytes, st

    P = mw.PoissonOperator(mra, prec)
    g1 = mw.FunctionTree(mra)
    mw.apply(prec, g1, P, f, precision=mw.FP64)
    f.rescale(1.0)  # marks the tree changed: the next apply uploads it again
    g2 = mw.FunctionTree(mra)
    mw.apply(prec, g2, P, f, precision=mw.FP64)
    a, b = g1.export(), g2.export()
    assert np.array_equal(a["idx"], b["idx"])
    assert np.abs(a["coefs"] - b["coefs"]).max() <= 1e-13 * np.abs(a["coefs"]).max()

    ref = oracle.apply(prec, mw.FunctionTree(mra), P, f)
    same, perm = match(b, ref)
    assert same
    mx, l2 = rel_errors(b["coefs"], ref["coefs"][perm])
    assert mx <= 1e-11 and l2 <= 1e-11

    # freed blocks go to the cache and serve the next tree of the same size
    live = mw.pinned_stats()["live_bytes"]
    del g2
    after = mw.pinned_stats()
    assert after["live_bytes"] < live and after["idle_bytes"] > 0
    g3 = mw.FunctionTree(mra)
    mw.apply(prec, g3, P, f, precision=mw.FP64)
    again = mw.pinned_stats()
    assert again["idle_bytes"] < after["idle_bytes"]
    assert np.array_equal(g3.export()["coefs"], b["coefs"]) or \
        np.abs(g3.export()["coefs"] - b["coefs"]).max() <= 1e-13 * np.abs(b["coefs"]).max()


def test_kernel_read_of_page_locked_inputs_equals_dma(gpu):
    # a page-locked input is read by a kernel through its device mapping (one
    # pass writing the FP64 array and the FP32 copy); MWGPU_H2D_DMA=1 takes
    # the copy engine and a separate conversion instead: the same device copy,
    # so the same results to the last bit, for fresh uploads and for new
    # values of a planned fixed-grid apply
    import os

    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    prec = 1e-4
    f = project(mra, prec, gaussian_sum(77, 5, (1.0, 100.0), (-5.0, 5.0)))
    assert mw.pinned_stats()["state"] == 1
    P = mw.PoissonOperator(mra, prec)
    grid = mw.FunctionTree(mra)
    mw.apply(prec, grid, P, f, precision=mw.FP64)
    res = {}
    for dma in (False, True):
        if dma:
            os.environ["MWGPU_H2D_DMA"] = "1"
        try:
            for form in (mw.FP64, mw.MIXED):
                f.rescale(1.0)  # uploaded again: the built level and the plan's update
                outs = []
                for cache in (False, True):
                    if not cache:
                        os.environ["MWH_NO_PLAN_CACHE"] = "1"
                    try:
                        g = mw.FunctionTree(mra)
                        mw.copy_grid(g, grid)
                        mw.apply(prec, g, P, f, max_iter=0, precision=form)
                        outs.append(g.export()["coefs"])
                    finally:
                        os.environ.pop("MWH_NO_PLAN_CACHE", None)
                res[(dma, form)] = outs
        finally:
            os.environ.pop("MWGPU_H2D_DMA", None)
    for form in (mw.FP64, mw.MIXED):
        for a, b in zip(res[(False, form)], res[(True, form)]):
            assert np.array_equal(a, b)
