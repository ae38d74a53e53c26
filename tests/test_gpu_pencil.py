"""The pencil contraction (k_pencil, order 7, terms of band width <= 4 on
levels without norm screening) against the item kernel alone
(MWGPU_NO_PENCIL=1) on the same levels: both are the mixed form, so the
results agree to the mixed form's accuracy (relative L2 <= 2e-6 between them,
each within 1e-5 of the FP64 form), with identical node-term and component
counts; the pencil kernel really takes part (its node-term count from
mwgpu_plan_pencil_info is positive and at most the level's).
"""
import ctypes as C
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
    f = project(mra, 1e-4, gaussian_sum(2026, 6, (1.0, 100.0), (-5.0, 5.0)))
    grid = mw.FunctionTree(mra)
    mw.apply(1e-4, grid, P, f, precision=mw.FP64)
    return mra, P, f, grid


def fixed(mra, P, f, grid, form, no_pencil=False, warps=None):
    if no_pencil:
        os.environ["MWGPU_NO_PENCIL"] = "1"
    if warps:
        os.environ["MWGPU_PENCIL_WARPS"] = str(warps)
    try:
        g = mw.FunctionTree(mra)
        mw.copy_grid(g, grid)
        st = mw.apply(1e-4, g, P, f, max_iter=0, precision=form)
    finally:
        os.environ.pop("MWGPU_NO_PENCIL", None)
        os.environ.pop("MWGPU_PENCIL_WARPS", None)
    return g.export()["coefs"], st


@pytest.mark.parametrize("warps", [8, 16])
def test_level_path(gpu, case, warps):
    # the pencil kernel with 8 consumer warps per CTA (two x values each) and
    # with 16 (one x value each): the same products, so the same sums up to
    # the order of FP32 additions
    mra, P, f, grid = case
    a, sa = fixed(mra, P, f, grid, mw.MIXED, warps=warps)
    b, sb = fixed(mra, P, f, grid, mw.MIXED, no_pencil=True)
    c, _ = fixed(mra, P, f, grid, mw.FP64)
    assert sa["node_terms"] == sb["node_terms"] and sa["components"] == sb["components"]
    rel = lambda x, y: np.linalg.norm(x - y) / np.linalg.norm(y)
    assert rel(a, b) <= 2e-6
    assert rel(a, c) <= 1e-5 and rel(b, c) <= 1e-5


def _plan_run(mra, P, f, grid, work, env, flags=1):
    """One planned mixed level over the output nodes `work` with the
    environment `env` set at plan creation: (coefficients of the work rows,
    node-terms, components, pencil node-terms, launches per execution, band
    widths of the operator by depth)."""
    L = mw.lib()
    os.environ.update(env)
    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    cfg.precision = mw.MIXED
    assert L.mwgpu_init(C.byref(ctx), C.byref(cfg)) == 0
    try:
        dop = C.c_void_p()
        assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-4, C.byref(dop)) == 0
        rows = C.c_int()
        assert L.mwgpu_operator_bandwidths(ctx, dop, C.byref(rows), None, None) == 0
        widths = np.zeros(P.desc().n_terms * rows.value * 5, dtype=np.int32)
        assert L.mwgpu_operator_bandwidths(ctx, dop, C.byref(rows), mw._pi(widths), None) == 0
        widths = widths.reshape(P.desc().n_terms, rows.value, 5)
        fx = f.export()
        fd = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), mw._pd(fx["coefs"]), mw._pd(fx["norms"]))
        dinp = C.c_void_p()
        assert L.mwgpu_upload_tree(ctx, C.byref(mra.desc()), C.byref(fd), C.byref(dinp)) == 0
        gx = grid.export()
        gd = mw.MwgpuTreeDesc(len(gx["child0"]), mw._pi(gx["idx"]), mw._pi(gx["child0"]), None, None)
        dout = C.c_void_p()
        assert L.mwgpu_create_tree(ctx, C.byref(mra.desc()), C.byref(gd), C.byref(dout)) == 0
        n = len(gx["child0"])
        work = np.ascontiguousarray(work, dtype=np.int32)
        PA1 = C.c_void_p * 1
        plan = C.c_void_p()
        sq = np.full(1, -1.0)
        rc = L.mwgpu_plan_create(ctx, dop, 1, PA1(dinp), PA1(dout), mw._pi(np.zeros(len(work), dtype=np.int32)), mw._pi(work),
                                 len(work), 1e-4, mw._pd(sq), flags, C.byref(plan))
        assert rc == 0, L.mwgpu_last_error(ctx).decode()
        for _ in range(2):
            assert L.mwgpu_plan_execute(ctx, plan, None) == 0
        st = mw.MwgpuLevelStats()
        assert L.mwgpu_plan_check(ctx, plan, C.byref(st)) == 0
        pnt, pms = C.c_ulonglong(), C.c_double()
        assert L.mwgpu_plan_pencil_info(plan, C.byref(pnt), C.byref(pms)) == 0
        lpe = C.c_ulonglong()
        assert L.mwgpu_plan_info(plan, None, None, None, None, None, C.byref(lpe)) == 0
        c = np.zeros((n, 8 * 512))
        assert L.mwgpu_download_tree(ctx, dout, mw._pd(c), None) == 0
        assert L.mwgpu_plan_destroy(ctx, plan) == 0
        return c[work], st.node_terms, st.components, pnt.value, lpe.value, widths
    finally:
        for k in env:
            os.environ.pop(k, None)
        L.mwgpu_destroy(ctx)


def test_plan_path(gpu, case):
    # "pencil": the plan configuration; "fill": the same with the item list
    # filled and compacted every execution (MWGPU_PLAN_FILL); "items": the
    # item kernel alone.  Where every term at the depth of every output node
    # is within the pencil kernel's band width, the plan leaves the item list
    # unfilled (fewer launches, the same bits); the work list of every node
    # may leave terms to the item kernel at some depths, that of the nodes at
    # depths whose band width is within the pencil kernel's none
    mra, P, f, grid = case
    gx = grid.export()
    allw = np.arange(len(gx["child0"]), dtype=np.int32)
    env = {"pencil": {}, "fill": {"MWGPU_PLAN_FILL": "1"}, "items": {"MWGPU_NO_PENCIL": "1"}}
    w = _plan_run(mra, P, f, grid, allw[:1], {"MWGPU_NO_PENCIL": "1"}, 0)[5]
    depth = gx["idx"][:, 0] - gx["idx"][:, 0].min()
    # a depth leaves nothing to the item kernel when every term there has band
    # width <= 4, or (below the roots, where the (s, s) block is left out) only
    # its (s, s) block wider and no other block in its band
    blocks = (w[:, :, 4] <= 4) | ((np.arange(w.shape[1]) > 0)[None, :] & (w[:, :, 1:4].max(axis=2) < 0))
    narrow = blocks.all(axis=0)[depth]
    fine = allw[narrow]
    assert len(fine) > 0
    # (the nodes of those depths alone without the transforms, which would
    # mix in the unset coefficients of the other nodes)
    for work, skips, flags in ((allw, len(fine) == len(allw), 1), (fine, True, 0)):
        out = {var: _plan_run(mra, P, f, grid, work, env[var], flags) for var in ("pencil", "fill", "items")}
        (a, nta, nca, pa, la, _), (b, ntb, ncb, pb, _, _) = out["pencil"], out["items"]
        assert nta == ntb and nca == ncb
        assert 0 < pa <= nta and pb == 0
        assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 2e-6
        fa, fnt, fnc, fpa, fl, _ = out["fill"]
        assert (fnt, fnc, fpa) == (nta, nca, pa)
        assert np.array_equal(fa, a)
        assert (la < fl) == skips
        if skips:
            assert pa == nta   # no term is left to the item kernel
def test_plan_autotuning(gpu, case):
    # MWGPU_PLAN_AUTOTUNE times the three schedules (pencil kernel with 8 or
    # 16 consumer warps + item kernel, item kernel alone) x 4 chunk lengths on
    # the level and keeps the fastest; the
    # result does not depend on the choice beyond the mixed form's accuracy
    mra, P, f, grid = case
    L = mw.lib()
    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    cfg.precision = mw.MIXED
    assert L.mwgpu_init(C.byref(ctx), C.byref(cfg)) == 0
    try:
        dop = C.c_void_p()
        assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-4, C.byref(dop)) == 0
        fx = f.export()
        fd = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), mw._pd(fx["coefs"]), mw._pd(fx["norms"]))
        dinp = C.c_void_p()
        assert L.mwgpu_upload_tree(ctx, C.byref(mra.desc()), C.byref(fd), C.byref(dinp)) == 0
        gx = grid.export()
        gd = mw.MwgpuTreeDesc(len(gx["child0"]), mw._pi(gx["idx"]), mw._pi(gx["child0"]), None, None)
        n = len(gx["child0"])
        PA1 = C.c_void_p * 1
        res = {}
        for flags in (1, 3):
            dout = C.c_void_p()
            assert L.mwgpu_create_tree(ctx, C.byref(mra.desc()), C.byref(gd), C.byref(dout)) == 0
            plan = C.c_void_p()
            sq = np.full(1, -1.0)
            rc = L.mwgpu_plan_create(ctx, dop, 1, PA1(dinp), PA1(dout), mw._pi(np.zeros(n, dtype=np.int32)), mw._pi(np.arange(n, dtype=np.int32)),
                                     n, 1e-4, mw._pd(sq), flags, C.byref(plan))
            assert rc == 0, L.mwgpu_last_error(ctx).decode()
            nc, chosen = C.c_int(16), C.c_int()
            items, sched, ms = (C.c_longlong * 16)(), (C.c_int * 16)(), (C.c_double * 16)()
            assert L.mwgpu_plan_tuning(plan, C.byref(nc), items, sched, ms, C.byref(chosen)) == 0
            if flags == 3:
                assert nc.value == 12 and sorted(set(sched[:12])) == [0, 1, 2]
                assert 0 <= chosen.value < 12 and ms[chosen.value] == min(ms[:12])
            else:
                assert nc.value == 0 and chosen.value == -1
            assert L.mwgpu_plan_execute(ctx, plan, None) == 0
            assert L.mwgpu_plan_check(ctx, plan, None) == 0
            c = np.zeros((n, 8 * 512))
            assert L.mwgpu_download_tree(ctx, dout, mw._pd(c), None) == 0
            assert L.mwgpu_plan_destroy(ctx, plan) == 0
            assert L.mwgpu_free_tree(ctx, dout) == 0
            res[flags] = c
        assert np.linalg.norm(res[3] - res[1]) / np.linalg.norm(res[1]) <= 2e-6
    finally:
        L.mwgpu_destroy(ctx)
