"""Learned output grid: the device-judged apply over a proposed grid
(mwgpu_apply_judged), the network's kernels against the CPU oracle
(oracle/mlp_oracle.py), and the learned apply against the plain one.

The judge is the split test itself, so whatever the proposal, the judged
result must equal the plain adaptive apply: the same topology (integer-exact)
and, in the FP64 form, the same coefficients to the last bits.  A proposal
that misses a refinement must say so (first_miss); the learned apply then keeps
the levels up to the miss and continues with the host TreeBuilder loop."""
import ctypes as C

import numpy as np
import pytest

import mrcpp_gb300 as mw
from cases import gaussian_sum, match, project, rel_errors
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

# two mixed-form contraction schedules of the same level (largest coefficient difference, relative)
MIXED_SCHED_TOL = 1e-6


def level_order(idx, child0, drop=(), extra=()):
    """Proposal arrays from a tree (idx, child0 of any node order): level by
    level, children in the order of their parents.  Nodes in `drop` lose their
    children; leaves in `extra` get 8 proposed children."""
    idx = np.asarray(idx).reshape(-1, 4)
    child0 = np.asarray(child0)
    roots = [i for i in range(len(idx)) if idx[i, 0] == idx[:, 0].min()]
    out_idx, out_c0, level_begin, src = [], [], [0], []
    cur = [("t", i) for i in roots]
    while cur:
        nxt = []
        for kind, i in cur:
            if kind == "t":
                out_idx.append(idx[i].tolist())
                src.append(i)
                node = idx[i]
                kids = None
                if child0[i] >= 0 and i not in drop:
                    kids = [("t", child0[i] + c) for c in range(8)]
                elif child0[i] < 0 and i in extra:
                    kids = [("x", (node[0] + 1, 2 * node[1] + (c & 1), 2 * node[2] + ((c >> 1) & 1), 2 * node[3] + (c >> 2))) for c in range(8)]
            else:
                out_idx.append(list(i))
                src.append(-1)
                kids = None
            out_c0.append(-1 if kids is None else -2)
            if kids:
                nxt.extend(kids)
        # child0 of this level's nodes: positions in the next level
        pos = len(out_idx)
        for j in range(level_begin[-1], len(out_idx)):
            if out_c0[j] == -2:
                out_c0[j] = pos
                pos += 8
        level_begin.append(len(out_idx))
        cur = nxt
    return (np.ascontiguousarray(np.array(out_idx, dtype=np.int32).ravel()), np.ascontiguousarray(np.array(out_c0, dtype=np.int32)),
            np.array(level_begin, dtype=np.int32), np.array(src))


class Judged:
    def __init__(self, mra, P, f, prec, precision):
        self.L = mw.lib()
        self.mra, self.prec = mra, prec
        self.ctx = C.c_void_p()
        cfg = mw.MwgpuConfig()
        cfg.precision = precision
        assert self.L.mwgpu_init(C.byref(self.ctx), C.byref(cfg)) == 0
        self.dop = C.c_void_p()
        assert self.L.mwgpu_upload_operator(self.ctx, C.byref(mra.desc()), C.byref(P.desc()), prec, C.byref(self.dop)) == 0
        fx = f.export()
        self.fx = fx
        d = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), mw._pd(fx["coefs"]), mw._pd(fx["norms"]))
        self.dinp = C.c_void_p()
        assert self.L.mwgpu_upload_tree(self.ctx, C.byref(mra.desc()), C.byref(d), C.byref(self.dinp)) == 0

    def run(self, pidx, pc0, lb):
        L = self.L
        n = len(pc0)
        d = mw.MwgpuTreeDesc(n, mw._pi(pidx), mw._pi(pc0), None, None)
        t = C.c_void_p()
        assert L.mwgpu_create_tree(self.ctx, C.byref(self.mra.desc()), C.byref(d), C.byref(t)) == 0
        flags = np.zeros(n, dtype=np.int32)
        miss = C.c_int()
        st = mw.MwgpuLevelStats()
        lb = np.ascontiguousarray(lb, dtype=np.int32)
        state0 = np.array([0.0, 0.0, -1.0])
        rc = L.mwgpu_apply_judged(self.ctx, self.dop, self.dinp, t, len(lb) - 1, mw._pi(lb), self.prec, 0, 0, mw._pd(state0), 1,
                                  mw._pi(flags), C.byref(miss), None, C.byref(st))
        assert rc == 0, L.mwgpu_last_error(self.ctx).decode()
        coefs = np.zeros((n, 8 * self.mra.kp1 ** 3))
        assert L.mwgpu_download_tree(self.ctx, t, mw._pd(coefs), None) == 0
        assert L.mwgpu_free_tree(self.ctx, t) == 0
        return flags, miss.value, coefs, st

    def close(self):
        self.L.mwgpu_destroy(self.ctx)


def _case(order=5, prec=1e-4, seed=21, n=4):
    mra = mw.MRA(box=(-20, 20), order=order, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, prec)
    f = project(mra, prec, gaussian_sum(seed, n, (2.0, 80.0), (-3.0, 3.0)))
    return mra, P, f


def _kept_tree(pidx, flags, coefs):
    keep = (flags & 1) == 1
    rows = {tuple(r): i for i, r in enumerate(pidx.reshape(-1, 4)[keep].tolist())}
    return keep, rows, coefs[keep]


@pytest.mark.parametrize("precision", [mw.FP64, mw.MIXED])
def test_judged_apply_equals_plain_for_exact_superset_and_deficient_proposals(gpu, precision):
    mra, P, f = _case()
    plain = mw.FunctionTree(mra)
    st_plain = mw.apply(1e-4, plain, P, f, precision=precision)
    gx = plain.export()
    J = Judged(mra, P, f, 1e-4, precision)
    try:
        tol = 1e-13
        # 1) the plain grid itself
        pidx, pc0, lb, src = level_order(gx["idx"], gx["child0"])
        flags, miss, coefs, st = J.run(pidx, pc0, lb)
        assert miss == -1
        assert (flags & 1).all() and ((flags & 2) > 0).sum() == (gx["child0"] >= 0).sum()
        assert st.node_terms == st_plain["node_terms"] and st.components == st_plain["components"]
        mx, _ = rel_errors(coefs, gx["coefs"][src])
        assert mx <= tol, mx
        # 2) a superset: extra children under some leaves are proposed and pruned
        leaves = [i for i in range(len(gx["child0"])) if gx["child0"][i] < 0][::5]
        pidx, pc0, lb, src = level_order(gx["idx"], gx["child0"], extra=set(leaves))
        flags, miss, coefs, st = J.run(pidx, pc0, lb)
        assert miss == -1
        keep = (flags & 1) == 1
        assert keep.sum() == len(gx["child0"])
        assert (src[keep] >= 0).all()
        mx, _ = rel_errors(coefs[keep], gx["coefs"][src[keep]])
        assert mx <= tol, mx
        assert st.node_terms == st_plain["node_terms"]
        # 3) a deficient proposal: a refined node of level 1 without children
        depth = gx["idx"].reshape(-1, 4)[:, 0] - gx["idx"].reshape(-1, 4)[:, 0].min()
        cand = [i for i in range(len(gx["child0"])) if gx["child0"][i] >= 0 and depth[i] == 1]
        if cand:
            pidx, pc0, lb, src = level_order(gx["idx"], gx["child0"], drop={cand[0]})
            flags, miss, coefs, st = J.run(pidx, pc0, lb)
            assert miss == 1
    finally:
        J.close()


def test_network_forward_and_gradient_against_oracle(gpu):
    L = mw.lib()
    ctx = C.c_void_p()
    assert L.mwgpu_init(C.byref(ctx), C.byref(mw.MwgpuConfig())) == 0
    try:
        p = mo.init_params(5)
        p[mo.OFF_B1:mo.OFF_W2] = 0.05
        net = C.c_void_p()
        assert L.mwgpu_mlp_create(ctx, mw._pf(p), C.byref(net)) == 0
        rng = np.random.default_rng(9)
        n = 1000   # not a multiple of the 128-sample tile
        x = rng.normal(size=(n, mo.F)).astype(np.float32)
        y = (rng.random(n) < 0.3).astype(np.float32)
        prob = np.zeros(n, dtype=np.float32)
        assert L.mwgpu_mlp_infer(ctx, net, mw._pf(x), n, mw._pf(prob)) == 0
        ref = mo.prob(p, x)
        assert np.abs(prob - ref).max() <= 2e-5, np.abs(prob - ref).max()
        g = np.zeros(mo.NPARAM, dtype=np.float32)
        loss = C.c_float()
        assert L.mwgpu_mlp_grad(ctx, net, mw._pf(x), mw._pf(y), n, 3.0, mw._pf(g), C.byref(loss)) == 0
        lref, gref = mo.loss_and_grad(p, x, y, 3.0)
        assert abs(loss.value - lref) <= 1e-5 * abs(lref)
        err = np.linalg.norm(g - gref) / np.linalg.norm(gref)
        assert err <= 1e-4, err
        # per block of parameters too
        for a, b in ((mo.OFF_W1, mo.OFF_B1), (mo.OFF_W2, mo.OFF_B2), (mo.OFF_W3, mo.OFF_B3)):
            e = np.linalg.norm(g[a:b] - gref[a:b]) / np.linalg.norm(gref[a:b])
            assert e <= 1e-4, (a, e)
        # BF16 copy = oracle rounding of the master weights
        wb = np.zeros(mo.NPARAM, dtype=np.uint16)
        assert L.mwgpu_mlp_get(ctx, net, None, wb.ctypes.data_as(C.POINTER(C.c_uint16))) == 0
        expect = (mo.bf16_round(p).view(np.uint32) >> 16).astype(np.uint16)
        assert np.array_equal(wb, expect)
        # training lowers the loss of a separable problem
        y2 = (x[:, 0] + 0.5 * x[:, 1] > 0.2).astype(np.float32)
        curve = np.zeros(20, dtype=np.float32)
        assert L.mwgpu_mlp_train(ctx, net, mw._pf(x), mw._pf(y2), n, 20, 256, 3e-3, 1.0, 7, mw._pf(curve)) == 0
        assert curve[-1] < 0.5 * curve[0], curve
        assert L.mwgpu_mlp_infer(ctx, net, mw._pf(x), n, mw._pf(prob)) == 0
        assert ((prob > 0.5) == (y2 > 0.5)).mean() > 0.95
        assert L.mwgpu_mlp_destroy(ctx, net) == 0
    finally:
        L.mwgpu_destroy(ctx)


def test_features_of_stored_nodes(gpu):
    """Features 0, 1, 3-7 of nodes the input tree stores, against the export."""
    mra, P, f = _case(order=5, prec=1e-3, seed=4, n=2)
    fx = f.export()
    idx = fx["idx"].reshape(-1, 4)
    x, _ = mw.grid_features(1e-3, f, P, f)
    fn = np.sqrt(max(f.square_norm, 0.0))
    own = np.sqrt((fx["norms"].reshape(-1, 8)[:, 1:] ** 2).sum(1))
    tot = np.sqrt((fx["norms"].reshape(-1, 8) ** 2).sum(1))
    depth = idx[:, 0] - idx[:, 0].min()
    assert np.allclose(x[:, 0], depth / 16.0)
    assert np.allclose(x[:, 1], np.log10(np.maximum(own / fn, 1e-30)) / 8.0, atol=1e-6)
    assert np.array_equal(x[:, 4:7], (idx[:, 1:4] & 1).astype(np.float32))
    assert np.array_equal(x[:, 7], np.where(fx["child0"] >= 0, 1.0, 0.5).astype(np.float32))
    assert (x[:, 2] >= np.log10(np.maximum(tot / fn, 1e-30)) / 8.0 - 1e-6).all()   # the band sum includes the node itself


def test_learned_apply_equals_plain_and_falls_back(gpu):
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-5)
    f = project(mra, 1e-5, gaussian_sum(31, 3, (1.0, 100.0), (-5.0, 5.0)))
    plain = mw.FunctionTree(mra)
    sp = mw.apply(1e-5, plain, P, f, precision=mw.MIXED)
    px = plain.export()
    # a network that refines everything down to a few levels proposes a superset
    # near the roots and misses below: the judge falls back to the plain apply
    p = np.zeros(mo.NPARAM, dtype=np.float32)
    p[mo.OFF_B3] = 10.0
    always = mw.GridNetwork(p)
    g1 = mw.FunctionTree(mra)
    st = mw.apply_learned(1e-5, g1, P, f, always, precision=mw.MIXED)
    same, perm = match(g1.export(), px)
    assert same
    # mixed form: the host-driven apply computes its first TreeBuilder level (no
    # norm screening) with the pencil contraction, the judged levels use the item
    # kernel; both sums are within the mixed-form accuracy of each other
    assert rel_errors(g1.export()["coefs"], px["coefs"][perm])[0] <= MIXED_SCHED_TOL
    # a network that refines nothing misses at level 0 (when the plain tree refines)
    q = np.zeros(mo.NPARAM, dtype=np.float32)
    q[mo.OFF_B3] = -10.0
    never = mw.GridNetwork(q)
    g2 = mw.FunctionTree(mra)
    st2 = mw.apply_learned(1e-5, g2, P, f, never, precision=mw.MIXED)
    same, perm = match(g2.export(), px)
    assert same
    if len(px["child0"]) > 8:
        assert st2["fallback"] == 1 and st2["first_miss"] == 0


def test_trained_network_against_plain_refinement(gpu):
    """The committed network on held-out densities of its training family: the
    learned apply gives the plain apply's tree (topology and coefficients) with
    fewer judged passes than the plain TreeBuilder has iterations."""
    from mrcpp_gb300.learned import train_grid as tg

    net = mw.GridNetwork.load()
    thr = float(net.meta["threshold"])
    full = int(net.meta["full_levels"])
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, tg.PREC)
    passes, iters = [], []
    for seed in range(tg.HELD_SEED0, tg.HELD_SEED0 + 6):
        f = mw.FunctionTree(mra)
        mw.project(tg.PREC, f, tg.density(seed))
        g0 = mw.FunctionTree(mra)
        sp = mw.apply(tg.PREC, g0, P, f, precision=mw.MIXED)
        g1 = mw.FunctionTree(mra)
        sl = mw.apply_learned(tg.PREC, g1, P, f, net, threshold=thr, full_levels=full, precision=mw.MIXED)
        a, b = g0.export(), g1.export()
        same, perm = match(b, a)
        assert same, seed
        mx, _ = rel_errors(b["coefs"], a["coefs"][perm])
        assert mx <= MIXED_SCHED_TOL, (seed, mx)
        passes.append(sl["apply"]["iterations"])
        iters.append(sp["iterations"])
    assert np.mean(passes) < np.mean(iters), (passes, iters)
