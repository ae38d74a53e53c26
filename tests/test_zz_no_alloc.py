"""mwgpu_apply_level_static: the level computation for callers that may not
allocate device memory while it runs (its scratch is a fixed device array).

Checked through the C-ABI against mwgpu_apply_level on the same level, on two
calls in a row, within the FP64 parity tolerance of the other GPU tests.
Runs last (file name) so that a failure here leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest

import mrcpp_gb300 as mw
from cases import project, unit_gaussian

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11


def _setup():
    L = mw.lib()
    L.mwgpu_apply_level_static.restype = C.c_int
    L.mwgpu_apply_level_static.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_double,
                                           C.c_double, C.POINTER(C.c_double), C.POINTER(mw.MwgpuLevelStats)]
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    f = project(mra, 1e-3, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    grid = mw.FunctionTree(mra)
    mw.apply(1e-3, grid, P, f, precision=mw.FP64)
    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    assert L.mwgpu_init(C.byref(ctx), C.byref(cfg)) == 0
    return L, mra, P, f, grid, ctx


def _upload(L, ctx, mra, P, f, grid, n_out_trees):
    dop = C.c_void_p()
    assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-3, C.byref(dop)) == 0
    fx = f.export()
    fd = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), mw._pd(fx["coefs"]), mw._pd(fx["norms"]))
    dinp = C.c_void_p()
    assert L.mwgpu_upload_tree(ctx, C.byref(mra.desc()), C.byref(fd), C.byref(dinp)) == 0
    gx = grid.export()
    gd = mw.MwgpuTreeDesc(len(gx["child0"]), mw._pi(gx["idx"]), mw._pi(gx["child0"]), None, None)
    outs = []
    for _ in range(n_out_trees):
        t = C.c_void_p()
        assert L.mwgpu_create_tree(ctx, C.byref(mra.desc()), C.byref(gd), C.byref(t)) == 0
        outs.append(t)
    return dop, dinp, outs, len(gx["child0"]), (fx, gx)


def _download(L, ctx, tree, n, K3):
    c = np.zeros((n, 8 * K3))
    assert L.mwgpu_download_tree(ctx, tree, mw._pd(c), None) == 0
    return c


def test_static_level_matches_allocating_level(gpu):
    L, mra, P, f, grid, ctx = _setup()
    try:
        dop, dinp, (out_a, out_b), n, keep = _upload(L, ctx, mra, P, f, grid, 2)
        K3 = mra.kp1 ** 3
        work = np.arange(n, dtype=np.int32)
        for precision, tol in ((mw.FP64, FP64_TOL),):
            assert L.mwgpu_set_precision(ctx, precision) == 0
            na = np.zeros((n, 8))
            sa = mw.MwgpuLevelStats()
            assert L.mwgpu_apply_level(ctx, dop, dinp, out_a, mw._pi(work), n, 1e-3, -1.0, mw._pd(na), C.byref(sa)) == 0
            ca = _download(L, ctx, out_a, n, K3)
            for call in range(2):
                nb = np.zeros((n, 8))
                sb = mw.MwgpuLevelStats()
                rc = L.mwgpu_apply_level_static(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, mw._pd(nb), C.byref(sb))
                assert rc == 0, L.mwgpu_last_error(ctx).decode()
                cb = _download(L, ctx, out_b, n, K3)
                err = np.linalg.norm(cb - ca) / np.linalg.norm(ca)
                assert err <= tol, (precision, call, err)
                assert np.abs(nb - na).max() <= tol * np.abs(na).max()
                assert sb.node_terms == sa.node_terms and sb.components == sa.components
    finally:
        L.mwgpu_destroy(ctx)


def test_static_level_rejects_what_it_cannot_do(gpu):
    L, mra, P, f, grid, ctx = _setup()
    try:
        dop, dinp, (out_b,), n, keep = _upload(L, ctx, mra, P, f, grid, 1)
        # the mixed form needs a work list whose size depends on the level: not offered here
        work = np.arange(n, dtype=np.int32)
        assert L.mwgpu_set_precision(ctx, mw.MIXED) == 0
        rc = L.mwgpu_apply_level_static(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, None)
        assert rc == 1 and b"FP64" in L.mwgpu_last_error(ctx)
        assert L.mwgpu_set_precision(ctx, mw.FP64) == 0
        # more nodes than the fixed scratch holds: rejected before any device work
        big = np.zeros(65537, dtype=np.int32)
        rc = L.mwgpu_apply_level_static(ctx, dop, dinp, out_b, mw._pi(big), len(big), 1e-3, -1.0, None, None)
        assert rc == 1 and b"65536" in L.mwgpu_last_error(ctx)
        # a fresh input tree has no GenNodes yet: when the bands need some, the
        # lookups miss and the call says so instead of allocating them
        work = np.arange(n, dtype=np.int32)
        rc = L.mwgpu_apply_level_static(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, None)
        msg = L.mwgpu_last_error(ctx)
        st = mw.MwgpuLevelStats()
        assert L.mwgpu_apply_level(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, C.byref(st)) == 0
        if st.gen_nodes > 0:
            assert rc == 1 and b"missing" in msg
        else:
            assert rc == 0
        # once they exist the same call succeeds
        assert L.mwgpu_apply_level_static(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, None) == 0
        if st.gen_nodes > 0:
            # GenNodes remade by a mixed-form level hold FP32-product values:
            # rejected until an FP64 level has remade them
            assert L.mwgpu_set_precision(ctx, mw.MIXED) == 0
            assert L.mwgpu_apply_level(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, None) == 0
            assert L.mwgpu_set_precision(ctx, mw.FP64) == 0
            rc = L.mwgpu_apply_level_static(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, None)
            assert rc == 1 and b"mixed" in L.mwgpu_last_error(ctx)
            assert L.mwgpu_apply_level(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, None) == 0
            assert L.mwgpu_apply_level_static(ctx, dop, dinp, out_b, mw._pi(work), n, 1e-3, -1.0, None, None) == 0
    finally:
        L.mwgpu_destroy(ctx)
