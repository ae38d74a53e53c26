"""GPU parity at the benchmark configurations as configured (seeds, sizes and
precisions of the reported workloads), both forms against the CPU oracle.

Each case asserts, for the FP64 and the mixed form:
  * the output topology equals the oracle's,
  * node-term and component counts equal the oracle's,
  * FP64: coefficients within 1e-11 of the largest coefficient;
    mixed: global relative L2 error <= 1e-5 against the oracle's coefficients,
  * the potential against its closed form (erf potential of each Gaussian for
    Poisson, the Yukawa potential of a Gaussian for Helmholtz) at seeded points,
    relative L2 error over the points <= 10 prec (measured about 1.4 prec).

Configurations:
  1  Poisson, interpolating k=5, [-20,20]^3, one normalised Gaussian exp(-10 r^2)
     centred at a seeded point of [-1,1]^3, prec 1e-3 (adaptive)
  2  Poisson, Legendre k=7, [-32,32]^3, 16 seeded Gaussians (exponents 1..100,
     centres [-5,5]^3), prec 1e-5: adaptive, then the fixed grid (maxIter = 0 on
     the oracle's output grid: the benchmark's level)
  3  Helmholtz mu=1, Legendre k=9, [-32,32]^3, 32 seeded Gaussians (exponents
     0.5..500, centres [-6,6]^3), prec 1e-6 (adaptive)
  4  8 of the 64 batch functions (1..32 Gaussians, exponents 0.1..1000, centres
     [-8,8]^3), k=7, prec 1e-5, one batched apply per form
"""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, rel_errors

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
MIXED_TOL = 1e-5
SEED = 2026


def coulomb(gs, x):
    """Closed-form potential int rho(y)/|x-y| dy of rho = sum c exp(-a |y-R|^2)."""
    v = 0.0
    for c, a, R in gs:
        d = float(np.linalg.norm(x - np.asarray(R)))
        v += c * (math.pi / a) ** 1.5 * (math.erf(math.sqrt(a) * d) / d if d > 1e-12 else 2.0 * math.sqrt(a / math.pi))
    return v


def yukawa(gs, x, mu):
    """Closed-form int exp(-mu|x-y|)/|x-y| rho(y) dy of the same Gaussian sum."""
    v = 0.0
    for c, a, R in gs:
        r = float(np.linalg.norm(x - np.asarray(R)))
        sb = math.sqrt(a)
        al = mu / (2.0 * sb)
        v += c * (math.pi / a) ** 1.5 * math.exp(mu * mu / (4.0 * a)) / (2.0 * r) * (
            math.exp(-mu * r) * math.erfc(al - sb * r) - math.exp(mu * r) * math.erfc(al + sb * r))
    return v


def potential_error(tree, fn, lo, hi, n=120, seed=7):
    rng = np.random.default_rng(seed)
    xs = rng.uniform(lo, hi, (n, 3))
    va = np.array([fn(x) for x in xs])
    vg = np.array([tree.evalf(x) for x in xs])
    return float(np.linalg.norm(vg - va) / np.linalg.norm(va))


def check(st, tree, ref, tol, what):
    gx = tree.export()
    same, perm = match(gx, ref)
    assert same, "%s: output topology differs from the oracle" % what
    assert st["node_terms"] == ref["node_terms"], (what, st["node_terms"], ref["node_terms"])
    assert st["components"] == ref["components"], (what, st["components"], ref["components"])
    mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
    if tol == FP64_TOL:
        assert mx <= tol, (what, mx)
    assert l2 <= tol, (what, l2)
    return l2


def both_forms(prec, mra, oper, f, ref, grid=None):
    """FP64 and mixed GPU applies (adaptive, or maxIter = 0 on `grid`) checked
    against the oracle result `ref`; returns the two trees."""
    out = {}
    for form, tol in ((mw.FP64, FP64_TOL), (mw.MIXED, MIXED_TOL)):
        g = mw.FunctionTree(mra)
        if grid is not None:
            mw.copy_grid(g, grid)
            st = mw.apply(prec, g, oper, f, max_iter=0, precision=form)
        else:
            st = mw.apply(prec, g, oper, f, precision=form)
        check(st, g, ref, tol, "FP64" if form == mw.FP64 else "mixed")
        out[form] = g
    return out


def test_config1_poisson_k5_seeded_centre(gpu):
    centre = tuple(float(x) for x in np.random.default_rng(SEED).uniform(-1.0, 1.0, 3))
    beta = 10.0
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    f = mw.FunctionTree(mra)
    gs = [((beta / math.pi) ** 1.5, beta, centre)]
    mw.project(1e-3, f, gs)
    ref = oracle.apply(1e-3, mw.FunctionTree(mra), P, f)
    trees = both_forms(1e-3, mra, P, f, ref)
    c = np.array(centre)
    for t in trees.values():
        assert potential_error(t, lambda x: coulomb(gs, x), c - 4.0, c + 4.0) <= 1e-2
        assert mw.dot(t, f) == pytest.approx(math.sqrt(2 * beta / math.pi), rel=1e-3)


@pytest.fixture(scope="module")
def config2():
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-5)
    gs = gaussian_sum(SEED, 16, (1.0, 100.0), (-5.0, 5.0))
    f = mw.FunctionTree(mra)
    mw.project(1e-5, f, gs)
    ref = oracle.apply(1e-5, mw.FunctionTree(mra), P, f)
    return mra, P, gs, f, ref


def test_config2_poisson_k7_adaptive(gpu, config2):
    mra, P, gs, f, ref = config2
    trees = both_forms(1e-5, mra, P, f, ref)
    for t in trees.values():
        assert potential_error(t, lambda x: coulomb(gs, x), -7.0, 7.0) <= 1e-4


def test_config2_poisson_k7_fixed_grid(gpu, config2):
    # the benchmark's level: maxIter = 0 onto the oracle's output grid (584
    # nodes, 464 244 node-terms, no norm screening); the GPU FP64 adaptive grid
    # the benchmark builds is the same grid
    mra, P, gs, f, ref_adaptive = config2
    grid = oracle.to_tree(ref_adaptive, mra)
    g0 = mw.FunctionTree(mra)
    mw.apply(1e-5, g0, P, f, precision=mw.FP64)
    same, _ = match(g0.export(), ref_adaptive)
    assert same, "the benchmark's GPU-built grid differs from the oracle's"
    gref = mw.FunctionTree(mra)
    mw.copy_grid(gref, grid)
    ref = oracle.apply(1e-5, gref, P, f, max_iter=0)
    assert ref["node_terms"] == 464244
    both_forms(1e-5, mra, P, f, ref, grid=grid)


def test_config3_helmholtz_k9(gpu):
    mra = mw.MRA(box=(-32, 32), order=9, basis=mw.LEGENDRE)
    H = mw.HelmholtzOperator(mra, 1.0, 1e-6)
    gs = gaussian_sum(SEED, 32, (0.5, 500.0), (-6.0, 6.0))
    f = mw.FunctionTree(mra)
    mw.project(1e-6, f, gs)
    ref = oracle.apply(1e-6, mw.FunctionTree(mra), H, f)
    trees = both_forms(1e-6, mra, H, f, ref)
    a, b = trees[mw.MIXED].export(), trees[mw.FP64].export()
    per_node = np.linalg.norm(a["coefs"] - b["coefs"], axis=1) / np.linalg.norm(b["coefs"], axis=1).max()
    assert per_node.max() <= MIXED_TOL
    for t in trees.values():
        assert potential_error(t, lambda x: yukawa(gs, x, 1.0), -8.0, 8.0) <= 1e-5


def test_config4_batch_functions(gpu):
    # the batch workload's functions 0, 8, ..., 56 (their own seeds and
    # Gaussian counts), applied as one batch per form
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-5)
    counts = np.random.default_rng(4044).integers(1, 33, 64)
    pick = list(range(0, 64, 8))
    fs = []
    for i in pick:
        f = mw.FunctionTree(mra)
        mw.project(1e-5, f, gaussian_sum(5000 + i, int(counts[i]), (0.1, 1000.0), (-8.0, 8.0)))
        fs.append(f)
    refs = [oracle.apply(1e-5, mw.FunctionTree(mra), P, f) for f in fs]
    for form, tol in ((mw.FP64, FP64_TOL), (mw.MIXED, MIXED_TOL)):
        outs = [mw.FunctionTree(mra) for _ in fs]
        st = mw.apply_batch(1e-5, outs, P, fs, precision=form)
        assert st["node_terms"] == sum(r["node_terms"] for r in refs)
        assert st["components"] == sum(r["components"] for r in refs)
        for t, r, i in zip(outs, refs, pick):
            gx = t.export()
            same, perm = match(gx, r)
            assert same, "function %d: topology differs from the oracle" % i
            mx, l2 = rel_errors(gx["coefs"], r["coefs"][perm])
            assert l2 <= tol, (i, l2)
            if form == mw.FP64:
                assert mx <= tol, (i, mx)
