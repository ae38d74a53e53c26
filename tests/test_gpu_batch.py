"""Batched apply: several functions through one operator with one device pass
per TreeBuilder iteration (mwgpu_apply_level_batch, mwgpu_transform_batch,
mwh_apply_batch).  Every output must equal the apply of its own pair: the FP64
form to the last bits of the summation order, the mixed form within the mixed
tolerance, both with the same output topology."""
import ctypes as C

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, project, rel_errors

pytestmark = pytest.mark.gpu

SAME_TOL = 1e-13   # batch vs separate, FP64: the same kernels on the same data
FP64_TOL = 1e-11   # FP64 vs oracle
MIXED_TOL = 1e-5


def _inputs(mra, prec, counts, seed0):
    return [project(mra, prec, gaussian_sum(seed0 + i, n, (1.0, 60.0), (-4.0, 4.0))) for i, n in enumerate(counts)]


def test_batch_fp64_equals_separate_applies(gpu):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-3)
    inps = _inputs(mra, 1e-3, (1, 4, 2, 7), 300)
    sep = []
    for f in inps:
        g = mw.FunctionTree(mra)
        st = mw.apply(1e-3, g, P, f, precision=mw.FP64)
        sep.append((g.export(), st))
    outs = [mw.FunctionTree(mra) for _ in inps]
    stb = mw.apply_batch(1e-3, outs, P, inps, precision=mw.FP64)
    for o, (ref, st) in zip(outs, sep):
        x = o.export()
        same, perm = match(x, ref)
        assert same, "batched output topology differs from the separate apply"
        mx, l2 = rel_errors(x["coefs"], ref["coefs"][perm])
        assert mx <= SAME_TOL, mx
    assert stb["node_terms"] == sum(st["node_terms"] for _, st in sep)
    assert stb["components"] == sum(st["components"] for _, st in sep)
    assert stb["out_nodes"] == sum(len(r["child0"]) for r, _ in sep)
    # and the largest one against the oracle
    big = int(np.argmax([len(r["child0"]) for r, _ in sep]))
    ref = oracle.apply(1e-3, mw.FunctionTree(mra), P, inps[big])
    same, perm = match(outs[big].export(), ref)
    assert same
    mx, _ = rel_errors(outs[big].export()["coefs"], ref["coefs"][perm])
    assert mx <= FP64_TOL, mx


def test_batch_mixed_against_fp64(gpu):
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-5)
    inps = _inputs(mra, 1e-5, (3, 1, 5), 700)
    ref = []
    for f in inps:
        g = mw.FunctionTree(mra)
        mw.apply(1e-5, g, P, f, precision=mw.FP64)
        ref.append(g.export())
    outs = [mw.FunctionTree(mra) for _ in inps]
    st = mw.apply_batch(1e-5, outs, P, inps, precision=mw.MIXED)
    assert st["node_terms"] > 0
    for o, r in zip(outs, ref):
        x = o.export()
        same, perm = match(x, r)
        assert same, "mixed batched topology differs from FP64"
        _, l2 = rel_errors(x["coefs"], r["coefs"][perm])
        assert l2 <= MIXED_TOL, l2


def _upload_input(L, ctx, mra, f):
    fx = f.export()
    d = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), mw._pd(fx["coefs"]), mw._pd(fx["norms"]))
    t = C.c_void_p()
    assert L.mwgpu_upload_tree(ctx, C.byref(mra.desc()), C.byref(d), C.byref(t)) == 0
    return t, fx


def _create_output(L, ctx, mra, grid):
    gx = grid.export()
    d = mw.MwgpuTreeDesc(len(gx["child0"]), mw._pi(gx["idx"]), mw._pi(gx["child0"]), None, None)
    t = C.c_void_p()
    assert L.mwgpu_create_tree(ctx, C.byref(mra.desc()), C.byref(d), C.byref(t)) == 0
    return t, gx


# mixed: the batched work list is chunked differently from the per-tree ones,
# so the FP32 partial sums are grouped differently (mixed tolerance)
@pytest.mark.parametrize("precision,tol", [(mw.FP64, SAME_TOL), (mw.MIXED, MIXED_TOL)])
def test_level_batch_interleaved_entries(gpu, precision, tol):
    """C-ABI: entries of three trees in shuffled order; norms come back in entry
    order; the batched level and transforms equal the per-tree calls."""
    L = mw.lib()
    mra = mw.MRA(box=(-20, 20), order=6, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    inps = _inputs(mra, 1e-4, (2, 5, 1), 900)
    grids = []
    for f in inps:
        g = mw.FunctionTree(mra)
        mw.apply(1e-4, g, P, f, precision=mw.FP64)
        grids.append(g)
    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    assert L.mwgpu_init(C.byref(ctx), C.byref(cfg)) == 0
    try:
        assert L.mwgpu_set_precision(ctx, precision) == 0
        dop = C.c_void_p()
        assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-4, C.byref(dop)) == 0
        fin_a = [_upload_input(L, ctx, mra, f)[0] for f in inps]
        fin_b = [_upload_input(L, ctx, mra, f)[0] for f in inps]
        outs_a, outs_b, sizes = [], [], []
        for g in grids:
            ta, gx = _create_output(L, ctx, mra, g)
            tb, _ = _create_output(L, ctx, mra, g)
            outs_a.append(ta)
            outs_b.append(tb)
            sizes.append(len(gx["child0"]))
        K8 = 8 * mra.kp1 ** 3
        # per tree, one level with all nodes (fixed grid, no norm screening)
        sep_norms, sep_nt = [], 0
        for t in range(3):
            work = np.arange(sizes[t], dtype=np.int32)
            nrm = np.zeros((sizes[t], 8))
            st = mw.MwgpuLevelStats()
            assert L.mwgpu_apply_level(ctx, dop, fin_a[t], outs_a[t], mw._pi(work), sizes[t], 1e-4, -1.0, mw._pd(nrm), C.byref(st)) == 0
            sep_norms.append(nrm)
            sep_nt += st.node_terms
            for d, ow in ((0, 0), (1, 1)):
                assert L.mwgpu_transform(ctx, outs_a[t], d, ow) == 0
        # batched: the same entries, shuffled across trees
        wt = np.concatenate([np.full(s, t, dtype=np.int32) for t, s in enumerate(sizes)])
        wn = np.concatenate([np.arange(s, dtype=np.int32) for s in sizes])
        perm = np.random.default_rng(5).permutation(len(wt))
        wt, wn = np.ascontiguousarray(wt[perm]), np.ascontiguousarray(wn[perm])
        n = len(wt)
        nb = np.zeros((n, 8))
        st = mw.MwgpuLevelStats()
        PA = C.c_void_p * 3
        sq = np.full(3, -1.0)
        rc = L.mwgpu_apply_level_batch(ctx, dop, 3, PA(*fin_b), PA(*outs_b), mw._pi(wt), mw._pi(wn), n, 1e-4, mw._pd(sq), mw._pd(nb),
                                       C.byref(st))
        assert rc == 0, L.mwgpu_last_error(ctx).decode()
        assert st.node_terms == sep_nt
        for j in range(n):
            ref = sep_norms[wt[j]][wn[j]]
            assert np.abs(nb[j] - ref).max() <= tol * max(np.abs(ref).max(), 1e-300) + 1e-300
        for d, ow in ((0, 0), (1, 1)):
            assert L.mwgpu_transform_batch(ctx, 3, PA(*outs_b), d, ow) == 0
        for t in range(3):
            ca = np.zeros((sizes[t], K8))
            cb = np.zeros((sizes[t], K8))
            assert L.mwgpu_download_tree(ctx, outs_a[t], mw._pd(ca), None) == 0
            assert L.mwgpu_download_tree(ctx, outs_b[t], mw._pd(cb), None) == 0
            assert np.linalg.norm(cb - ca) <= tol * np.linalg.norm(ca), t
        # a tree given twice is refused
        rc = L.mwgpu_apply_level_batch(ctx, dop, 2, PA(fin_b[0], fin_b[0]), PA(outs_b[0], outs_b[1]), mw._pi(wt), mw._pi(wn), 1, 1e-4,
                                       mw._pd(sq), None, None)
        assert rc == 1 and b"distinct" in L.mwgpu_last_error(ctx)
    finally:
        L.mwgpu_destroy(ctx)


def _download(L, ctx, tree, n, K8):
    c = np.zeros((n, K8))
    assert L.mwgpu_download_tree(ctx, tree, mw._pd(c), None) == 0
    return c


@pytest.mark.parametrize("precision", [mw.FP64, mw.MIXED])
def test_plan_graph_replays_the_level(gpu, precision):
    """A plan (GenNodes, work list, persistent contraction, reduction and both
    transforms captured as one CUDA graph) gives the result of the level calls,
    gives it again on every execution, follows new input coefficients, and
    holds its trees against structural changes."""
    L = mw.lib()
    mra = mw.MRA(box=(-20, 20), order=6, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    inps = _inputs(mra, 1e-4, (3, 1, 4), 1100)
    grids = []
    for f in inps:
        g = mw.FunctionTree(mra)
        mw.apply(1e-4, g, P, f, precision=mw.FP64)
        grids.append(g)
    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    assert L.mwgpu_init(C.byref(ctx), C.byref(cfg)) == 0
    plan = C.c_void_p()
    try:
        dop = C.c_void_p()
        assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-4, C.byref(dop)) == 0
        ups = [_upload_input(L, ctx, mra, f) for f in inps]
        fin_a = [u[0] for u in ups]
        fin_b = [_upload_input(L, ctx, mra, f)[0] for f in inps]
        outs_a, outs_b, sizes = [], [], []
        for g in grids:
            ta, gx = _create_output(L, ctx, mra, g)
            tb, _ = _create_output(L, ctx, mra, g)
            outs_a.append(ta)
            outs_b.append(tb)
            sizes.append(len(gx["child0"]))
        K8 = 8 * mra.kp1 ** 3
        # reference: FP64 level calls per tree + transforms
        assert L.mwgpu_set_precision(ctx, mw.FP64) == 0
        nt_ref = 0
        for t in range(3):
            work = np.arange(sizes[t], dtype=np.int32)
            st = mw.MwgpuLevelStats()
            assert L.mwgpu_apply_level(ctx, dop, fin_a[t], outs_a[t], mw._pi(work), sizes[t], 1e-4, -1.0, None, C.byref(st)) == 0
            nt_ref += st.node_terms
            assert L.mwgpu_transform(ctx, outs_a[t], 0, 0) == 0
            assert L.mwgpu_transform(ctx, outs_a[t], 1, 1) == 0
        ref = [_download(L, ctx, outs_a[t], sizes[t], K8) for t in range(3)]
        tol = SAME_TOL if precision == mw.FP64 else MIXED_TOL

        def close(res, tol):
            for t in range(3):
                err = np.linalg.norm(res[t] - ref[t]) / np.linalg.norm(ref[t])
                assert err <= tol, (t, err)

        assert L.mwgpu_set_precision(ctx, precision) == 0
        wt = np.concatenate([np.full(s, t, dtype=np.int32) for t, s in enumerate(sizes)])
        wn = np.concatenate([np.arange(s, dtype=np.int32) for s in sizes])
        PA = C.c_void_p * 3
        sq = np.full(3, -1.0)
        rc = L.mwgpu_plan_create(ctx, dop, 3, PA(*fin_b), PA(*outs_b), mw._pi(wt), mw._pi(wn), len(wt), 1e-4, mw._pd(sq), 3, C.byref(plan))
        assert rc == 0, L.mwgpu_last_error(ctx).decode()
        first = [_download(L, ctx, outs_b[t], sizes[t], K8) for t in range(3)]
        close(first, tol)
        runs = []
        for _ in range(2):
            st = mw.MwgpuLevelStats()
            assert L.mwgpu_plan_execute(ctx, plan, C.byref(st)) == 0, L.mwgpu_last_error(ctx).decode()
            assert st.node_terms == nt_ref
            runs.append([_download(L, ctx, outs_b[t], sizes[t], K8) for t in range(3)])
        for t in range(3):
            assert np.array_equal(runs[0][t], runs[1][t]), "graph executions differ"
            assert np.linalg.norm(runs[0][t] - first[t]) <= 1e-13 * np.linalg.norm(first[t])
        per, grid, ncand, launches = C.c_longlong(), C.c_int(), C.c_int(8), C.c_ulonglong()
        cand_items = (C.c_longlong * 8)()
        cand_ms = (C.c_double * 8)()
        assert L.mwgpu_plan_info(plan, C.byref(per), C.byref(grid), C.byref(ncand), cand_items, cand_ms, C.byref(launches)) == 0
        assert launches.value > 0
        if precision == mw.MIXED:
            assert per.value > 0 and grid.value > 0 and ncand.value == 4
            assert per.value in list(cand_items)[:4]
        # the trees are held by the plan
        work = np.arange(sizes[0], dtype=np.int32)
        assert L.mwgpu_apply_level(ctx, dop, fin_b[0], outs_b[0], mw._pi(work), sizes[0], 1e-4, -1.0, None, None) == 1
        assert b"plan" in L.mwgpu_last_error(ctx)
        assert L.mwgpu_tree_clear_generated(ctx, fin_b[1]) == 1
        # new input values, same topology: the output follows (linearity)
        for t in range(3):
            fx = ups[t][1]
            c2 = np.ascontiguousarray(2.0 * fx["coefs"])
            n2 = np.ascontiguousarray(2.0 * fx["norms"])
            assert L.mwgpu_tree_update_coefs(ctx, fin_b[t], mw._pd(c2), mw._pd(n2)) == 0
        assert L.mwgpu_plan_execute(ctx, plan, None) == 0
        assert L.mwgpu_plan_check(ctx, plan, None) == 0
        for t in range(3):
            x = _download(L, ctx, outs_b[t], sizes[t], K8)
            assert np.linalg.norm(x - 2.0 * runs[0][t]) <= 1e-12 * np.linalg.norm(x) + (0 if precision == mw.FP64 else 1e-6 * np.linalg.norm(x))
        assert L.mwgpu_plan_destroy(ctx, plan) == 0
        plan = None
        assert L.mwgpu_tree_clear_generated(ctx, fin_b[1]) == 0
    finally:
        if plan:
            L.mwgpu_plan_destroy(ctx, plan)
        L.mwgpu_destroy(ctx)


def test_plan_gen_node_families_are_bit_identical(gpu, monkeypatch):
    """Mixed-form plans compute their GenNodes per parent (k_gen_family32: the
    children of a parent share its x and y steps); the level they leave equals,
    bit for bit, the one of a plan with one GenNode per CTA
    (MWGPU_GEN_PER_NODE at plan creation).  Same chunking (no autotuning)."""
    L = mw.lib()
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    inps = _inputs(mra, 1e-4, (4, 2), 1200)
    grids = []
    for f in inps:
        g = mw.FunctionTree(mra)
        mw.apply(1e-4, g, P, f, precision=mw.FP64)
        grids.append(g)
    ctx = C.c_void_p()
    assert L.mwgpu_init(C.byref(ctx), C.byref(mw.MwgpuConfig())) == 0
    try:
        dop = C.c_void_p()
        assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-4, C.byref(dop)) == 0
        assert L.mwgpu_set_precision(ctx, mw.MIXED) == 0
        K8 = 8 * mra.kp1 ** 3
        res, gen = {}, {}
        for per_node in (True, False):
            if per_node:
                monkeypatch.setenv("MWGPU_GEN_PER_NODE", "1")
            else:
                monkeypatch.delenv("MWGPU_GEN_PER_NODE", raising=False)
            fin = [_upload_input(L, ctx, mra, f)[0] for f in inps]
            outs, sizes = [], []
            for g in grids:
                t, gx = _create_output(L, ctx, mra, g)
                outs.append(t)
                sizes.append(len(gx["child0"]))
            wt = np.concatenate([np.full(s, t, dtype=np.int32) for t, s in enumerate(sizes)])
            wn = np.concatenate([np.arange(s, dtype=np.int32) for s in sizes])
            PA = C.c_void_p * len(inps)
            sq = np.full(len(inps), -1.0)
            plan = C.c_void_p()
            rc = L.mwgpu_plan_create(ctx, dop, len(inps), PA(*fin), PA(*outs), mw._pi(wt), mw._pi(wn), len(wt), 1e-4, mw._pd(sq),
                                     1, C.byref(plan))  # MWGPU_PLAN_TRANSFORMS, no autotuning
            assert rc == 0, L.mwgpu_last_error(ctx).decode()
            st = mw.MwgpuLevelStats()
            assert L.mwgpu_plan_execute(ctx, plan, C.byref(st)) == 0, L.mwgpu_last_error(ctx).decode()
            gen[per_node] = st.gen_nodes
            res[per_node] = [_download(L, ctx, outs[t], sizes[t], K8) for t in range(len(inps))]
            assert L.mwgpu_plan_destroy(ctx, plan) == 0
        assert gen[True] == gen[False] > 0
        for a, b in zip(res[True], res[False]):
            assert np.array_equal(a, b)
    finally:
        L.mwgpu_destroy(ctx)


def test_level_gen_node_families_are_bit_identical(gpu, monkeypatch):
    """Mixed-form levels form GenNode families on the device (k_fam_* kernels,
    then k_gen_family32, ancestors may be GenNodes of earlier levels); the
    adaptive apply equals, bit for bit, the one with one GenNode per CTA."""
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = _inputs(mra, 1e-4, (5,), 1300)[0]
    res = {}
    for per_node in (True, False):
        if per_node:
            monkeypatch.setenv("MWGPU_GEN_PER_NODE", "1")
        else:
            monkeypatch.delenv("MWGPU_GEN_PER_NODE", raising=False)
        g = mw.FunctionTree(mra)
        st = mw.apply(1e-4, g, P, f, precision=mw.MIXED)
        res[per_node] = (g.export(), st["gen_nodes"])
    (a, ga), (b, gb) = res[True], res[False]
    assert ga == gb > 0
    assert np.array_equal(a["idx"], b["idx"])
    assert np.array_equal(a["coefs"], b["coefs"])


def test_plan_work_list_outgrowing_its_capacity_is_reported(gpu):
    """A mixed plan of a screened level (a positive output square norm) sizes
    its work list from the screening at plan time.  Input values a million
    times larger let far more component products pass the same threshold (set
    1e4 times above the apply's here): the
    list outgrows its buffer, the fill writes nothing beyond it, the passes
    that read the items stop at its end, and execute returns MWGPU_ERR_OOM
    (2); the context stays usable."""
    L = mw.lib()
    mra = mw.MRA(box=(-20, 20), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = _inputs(mra, 1e-4, (3,), 2200)[0]
    grid = mw.FunctionTree(mra)
    mw.apply(1e-4, grid, P, f, precision=mw.FP64)
    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    cfg.precision = mw.MIXED
    assert L.mwgpu_init(C.byref(ctx), C.byref(cfg)) == 0
    try:
        dop = C.c_void_p()
        assert L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(P.desc()), 1e-4, C.byref(dop)) == 0
        dinp, fx = _upload_input(L, ctx, mra, f)
        dout, gx = _create_output(L, ctx, mra, grid)
        n = len(gx["child0"])
        PA1 = C.c_void_p * 1
        plan = C.c_void_p()
        # a square norm 1e8 times that of the result: a screening threshold 1e4
        # times higher than the apply's, which keeps few products at plan time
        sq = np.full(1, grid.square_norm * 1e8)
        assert sq[0] > 0.0
        rc = L.mwgpu_plan_create(ctx, dop, 1, PA1(dinp), PA1(dout), mw._pi(np.zeros(n, dtype=np.int32)), mw._pi(np.arange(n, dtype=np.int32)),
                                 n, 1e-4, mw._pd(sq), 1, C.byref(plan))
        assert rc == 0, L.mwgpu_last_error(ctx).decode()
        st = mw.MwgpuLevelStats()
        assert L.mwgpu_plan_execute(ctx, plan, C.byref(st)) == 0
        screened = st.node_terms
        big = np.ascontiguousarray(fx["coefs"] * 1e6)
        assert L.mwgpu_tree_update_coefs(ctx, dinp, mw._pd(big), None) == 0
        rc = L.mwgpu_plan_execute(ctx, plan, C.byref(st))
        assert rc == 2, (rc, L.mwgpu_last_error(ctx).decode())
        assert "outgrew" in L.mwgpu_last_error(ctx).decode()
        assert L.mwgpu_plan_destroy(ctx, plan) == 0
        # the context still computes: the same level without the plan
        assert L.mwgpu_sync(ctx) == 0
        st2 = mw.MwgpuLevelStats()
        assert L.mwgpu_apply_level(ctx, dop, dinp, dout, mw._pi(np.arange(n, dtype=np.int32)), n, 1e-4, float(sq[0]), None, C.byref(st2)) == 0
        assert st2.node_terms > 1.25 * screened
    finally:
        L.mwgpu_destroy(ctx)
