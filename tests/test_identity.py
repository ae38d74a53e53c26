"""Identity convolution: the reference's known-answer test
tests/operators/identity_convolution.cpp:117-140 (3D).

IdentityConvolution(MRA, 1e-4) applied at 1e-3 to the unit Gaussian of
exponent 1e4 at (-0.2, 0.5, 1.0), projected at 1e-3 in the test world (scale
1, corner (-1, 0, 1), 1 x 2 x 3 boxes, interpolating order 5): the output is
no deeper and has no more nodes than the input, and integrates to the input's
integral within 1e-3.  CPU: the oracle; GPU: both forms, also node by node
against the oracle.
"""
import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import match, rel_errors, unit_gaussian


def setup():
    mra = mw.MRA(order=5, basis=mw.INTERPOLATING, scale=1, corner=(-1, 0, 1), nbox=(1, 2, 3), sf=1.0)
    f = mw.FunctionTree(mra)
    mw.project(1e-3, f, unit_gaussian(1e4, (-0.2, 0.5, 1.0)), grid=False)
    return mra, mw.IdentityConvolution(mra, 1e-4), f


def check(g, f):
    gx, fx = g.export(), f.export()
    assert gx["idx"][:, 0].max() <= fx["idx"][:, 0].max()
    assert g.n_nodes <= f.n_nodes
    assert g.integrate() == pytest.approx(f.integrate(), rel=1e-3)


def test_oracle_identity_convolution():
    mra, I, f = setup()
    assert I.size() == 1
    g = oracle.to_tree(oracle.apply(1e-3, mw.FunctionTree(mra), I, f, count_terms=False), mra)
    check(g, f)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [mw.FP64, mw.MIXED])
def test_gpu_identity_convolution(gpu, precision):
    mra, I, f = setup()
    g = mw.FunctionTree(mra)
    st = mw.apply(1e-3, g, I, f, precision=precision)
    check(g, f)
    ref = oracle.apply(1e-3, mw.FunctionTree(mra), I, f)
    same, perm = match(g.export(), ref)
    assert same
    mx, l2 = rel_errors(g.export()["coefs"], ref["coefs"][perm])
    if precision == mw.FP64:
        assert mx <= 1e-11, mx
        assert st["node_terms"] == ref["node_terms"]
    else:
        assert l2 <= 1e-5, l2
