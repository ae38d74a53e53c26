"""The precTrees form of apply (src/treebuilders/apply.h:43, apply.cpp:214-251)
on the CPU: the host precision function (mwh_prec_factors) against a numpy
restatement of makeMaxSquareNorms for nodes the precision tree holds, against
the orthonormality of the two-scale transform for nodes it lacks (generated
for their norm), and the oracle's precTrees path against its plain path.
"""
import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, project, unit_gaussian


@pytest.fixture(scope="module")
def trees():
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    f = project(mra, 1e-3, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    h = project(mra, 1e-3, gaussian_sum(11, 3, (1.0, 30.0), (-6.0, 6.0)))
    return mra, f, h


def max_square_norms(x):
    """MWNode::setMaxSquareNorm (MWNode.cpp:1257-1269) over a flat export:
    the largest 2^(3n) |node|^2 over the node and its descendants."""
    n = len(x["child0"])
    sq = (x["norms"] ** 2).sum(axis=1)
    msq = np.ldexp(1.0, 3 * x["idx"][:, 0]) * sq
    for i in range(n - 1, -1, -1):  # breadth-first export: children after parents
        c0 = x["child0"][i]
        if c0 >= 0:
            msq[i] = max(msq[i], msq[c0:c0 + 8].max())
    return msq, sq


def children(idx):
    n, l = idx[0], np.asarray(idx[1:])
    return np.array([[n + 1] + list(2 * l + np.array([c & 1, (c >> 1) & 1, (c >> 2) & 1])) for c in range(8)], dtype=np.int32)


def test_factors_of_held_nodes(trees):
    mra, f, h = trees
    x = f.export()
    msq, _ = max_square_norms(x)
    fac = mw.prec_factors([f], x["idx"])
    with np.errstate(divide="ignore"):  # nodes where f is exactly zero: precFac = inf
        want = 1.0 / np.sqrt(msq)
    np.testing.assert_allclose(fac, want, rtol=1e-14, atol=0)
    # two trees: 1 / the larger norm
    y = h.export()
    fh = mw.prec_factors([f, h], x["idx"])
    np.testing.assert_allclose(fh, np.minimum(fac, mw.prec_factors([h], x["idx"])), rtol=0, atol=0)
    # no trees: 1
    assert np.all(mw.prec_factors([], x["idx"][:5]) == 1.0)
    assert len(y["idx"]) > 8


def test_factors_of_generated_nodes(trees):
    # a leaf's 8 children (generated from it) carry its whole square norm, and
    # so do its 64 grandchildren (generated from generated nodes)
    mra, f, h = trees
    x = f.export()
    _, sq = max_square_norms(x)
    leaves = np.where(x["child0"] < 0)[0]
    big = leaves[np.argsort(-sq[leaves])[:6]]
    for i in big:
        kids = children(x["idx"][i])
        fac = mw.prec_factors([f], kids)
        s1 = (1.0 / fac ** 2 / np.ldexp(1.0, 3 * kids[:, 0])).sum()
        assert s1 == pytest.approx(sq[i], rel=1e-12)
        grand = np.concatenate([children(k) for k in kids])
        fac2 = mw.prec_factors([f], grand)
        s2 = (1.0 / fac2 ** 2 / np.ldexp(1.0, 3 * grand[:, 0])).sum()
        assert s2 == pytest.approx(sq[i], rel=1e-12)
    # the precision tree is read only
    assert f.n_nodes == len(x["child0"])


def test_zero_tree_gives_infinite_factor(trees):
    mra, f, h = trees
    z = project(mra, 1e-3, [(0.0, 1.0, (0.0, 0.0, 0.0))])
    fac = mw.prec_factors([z], z.export()["idx"])
    assert np.all(np.isinf(fac))


def test_oracle_prec_trees(trees):
    mra, f, h = trees
    P = mw.PoissonOperator(mra, 1e-3)
    plain = oracle.apply(1e-3, mw.FunctionTree(mra), P, f)
    empty = oracle.apply(1e-3, mw.FunctionTree(mra), P, f, prec_trees=[])
    assert np.array_equal(plain["idx"], empty["idx"]) and np.array_equal(plain["coefs"], empty["coefs"])
    assert plain["node_terms"] == empty["node_terms"] and plain["components"] == empty["components"]
    scaled = oracle.apply(1e-3, mw.FunctionTree(mra), P, f, prec_trees=[f])
    # precFac = 1 / max norm of f: a different grid from the plain apply
    assert scaled["n_nodes"] != plain["n_nodes"]
    # the potential is still the Coulomb potential of f, to the (locally scaled) precision
    t = mw.FunctionTree(mra)
    t.load_flat(scaled["idx"], scaled["child0"], scaled["coefs"])
    beta = 10.0
    assert mw.dot(t, f) == pytest.approx(np.sqrt(2 * beta / np.pi), rel=1e-3)
