"""GPU parity of the precTrees form of apply (src/treebuilders/apply.h:43,
apply.cpp:214-251) against the oracle's restatement: the precision of every
output node scaled by precFac = 1 / max sqrt(maxSquareNorm) of the precision
trees, in the screening threshold (ConvolutionCalculator.cpp:244-245) and the
split test (WaveletAdaptor.h:51-54).

Both forms: identical topology, node-term and component counts; FP64
coefficients within 1e-11 of the largest, mixed within 1e-5 (global relative
L2).  Each case changes the grid against the plain apply.
"""
import ctypes as C

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, project, rel_errors, unit_gaussian

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
MIXED_TOL = 1e-5


def check_both(prec, mra, oper, f, prec_trees):
    ref = oracle.apply(prec, mw.FunctionTree(mra), oper, f, prec_trees=prec_trees)
    plain = oracle.apply(prec, mw.FunctionTree(mra), oper, f, count_terms=False)
    assert ref["n_nodes"] != plain["n_nodes"], "precFac does not change the grid in this case"
    for form, tol in ((mw.FP64, FP64_TOL), (mw.MIXED, MIXED_TOL)):
        g = mw.FunctionTree(mra)
        st = mw.apply(prec, g, oper, f, prec_trees=prec_trees, precision=form)
        gx = g.export()
        same, perm = match(gx, ref)
        assert same, "topology differs from the oracle (%s)" % form
        assert st["node_terms"] == ref["node_terms"], (form, st["node_terms"], ref["node_terms"])
        assert st["components"] == ref["components"], (form, st["components"], ref["components"])
        mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
        assert l2 <= tol, (form, l2)
        if form == mw.FP64:
            assert mx <= tol, (form, mx)
    return ref


def test_prec_trees_poisson_k5(gpu):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    f = project(mra, 1e-3, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    h = project(mra, 1e-3, gaussian_sum(11, 3, (1.0, 30.0), (-6.0, 6.0)))
    check_both(1e-3, mra, P, f, [f])
    check_both(1e-3, mra, P, f, [f, h])


def test_prec_trees_poisson_k7_positional(gpu):
    # order 7 (the first iteration runs the pencil contraction, the screened
    # iterations the item kernel with per-node thresholds); the reference's
    # argument order apply(prec, out, oper, inp, precTrees, maxIter, absPrec)
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-5)
    gs = gaussian_sum(2026, 4, (1.0, 100.0), (-5.0, 5.0))
    f = project(mra, 1e-5, gs)
    ref = check_both(1e-5, mra, P, f, [f])
    g = mw.FunctionTree(mra)
    mw.apply(1e-5, g, P, f, [f], -1, False)
    same, _ = match(g.export(), ref)
    assert same


def test_zero_prec_tree_stops_refinement(gpu):
    # precFac = inf everywhere: no split after the first iteration
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    f = project(mra, 1e-3, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    z = project(mra, 1e-3, [(0.0, 1.0, (0.0, 0.0, 0.0))])
    ref = oracle.apply(1e-3, mw.FunctionTree(mra), P, f, prec_trees=[z])
    g = mw.FunctionTree(mra)
    st = mw.apply(1e-3, g, P, f, prec_trees=[z], precision=mw.FP64)
    assert st["iterations"] == ref["iterations"] == 1
    same, perm = match(g.export(), ref)
    assert same and st["node_terms"] == ref["node_terms"]


def test_scaled_level_rejects_bad_factors(gpu):
    L = mw.lib()
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    f = project(mra, 1e-3, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    assert L.mwgpu_init(C.byref(ctx), C.byref(cfg)) == 0
    try:
        dop = C.c_void_p()
        assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-3, C.byref(dop)) == 0
        fx = f.export()
        fd = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), mw._pd(fx["coefs"]), mw._pd(fx["norms"]))
        dinp = C.c_void_p()
        assert L.mwgpu_upload_tree(ctx, C.byref(mra.desc()), C.byref(fd), C.byref(dinp)) == 0
        gd = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), None, None)
        dout = C.c_void_p()
        assert L.mwgpu_create_tree(ctx, C.byref(mra.desc()), C.byref(gd), C.byref(dout)) == 0
        n = len(fx["child0"])
        work = np.arange(n, dtype=np.int32)
        for bad in (-1.0, np.nan):
            fac = np.ones(n)
            fac[n // 2] = bad
            rc = L.mwgpu_apply_level_scaled(ctx, dop, dinp, dout, mw._pi(work), n, 1e-3, 1.0, mw._pd(fac), None, None)
            assert rc == 1 and b"factors" in L.mwgpu_last_error(ctx)
        # factors of 1 give the plain level, bit for bit
        a, b = np.zeros((n, 8)), np.zeros((n, 8))
        assert L.mwgpu_apply_level(ctx, dop, dinp, dout, mw._pi(work), n, 1e-3, 1.0, mw._pd(a), None) == 0
        fac = np.ones(n)
        assert L.mwgpu_apply_level_scaled(ctx, dop, dinp, dout, mw._pi(work), n, 1e-3, 1.0, mw._pd(fac), mw._pd(b), None) == 0
        assert np.array_equal(a, b)
    finally:
        L.mwgpu_destroy(ctx)
