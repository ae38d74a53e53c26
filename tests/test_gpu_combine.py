"""GPU parity of addition and multiplication (mwgpu_combine_level under the
host TreeBuilder loop) against the CPU oracle: identical adaptive grids,
FP64 coefficients within 1e-12 of the largest."""
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, project, rel_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("basis,order", [(mw.INTERPOLATING, 5), (mw.LEGENDRE, 7)])
@pytest.mark.parametrize("op", [0, 1])
def test_combine_gpu_vs_oracle(gpu, basis, order, op):
    mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
    A = project(mra, 1e-5, gaussian_sum(51, 3, (0.5, 20.0), (-1.5, 1.5)))
    B = project(mra, 1e-5, gaussian_sum(52, 2, (1.0, 10.0), (-1.0, 1.0)))
    terms = [(1.5, A), (-0.5, B)] if op == 0 else [(2.0, A), (1.0, B)]
    g = mw.FunctionTree(mra)
    st = (mw.add if op == 0 else mw.multiply)(1e-5, g, terms)
    ref = oracle.combine(op, 1e-5, mw.FunctionTree(mra), terms)
    gx = g.export()
    same, perm = match(gx, ref)
    assert same, "adaptive grid differs from the oracle"
    mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
    assert mx <= 1e-12 and l2 <= 1e-12, (mx, l2)
    assert st["iterations"] == ref["iterations"]
    assert g.square_norm == pytest.approx(ref["square_norm"], rel=1e-12)


def test_combine_signature_forms(gpu):
    # add(prec, out, a, A, b, B) and multiply(prec, out, c, A, B) (add.h / multiply.h)
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    A = project(mra, 1e-4, gaussian_sum(53, 2, (1.0, 5.0), (-1.0, 1.0)))
    B = project(mra, 1e-4, gaussian_sum(54, 2, (1.0, 5.0), (-1.0, 1.0)))
    s1, s2 = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.add(1e-4, s1, 1.0, A, -1.0, B)
    mw.add(1e-4, s2, [(1.0, A), (-1.0, B)])
    assert match(s1.export(), {"idx": s2.export()["idx"]})[0]
    p1, p2 = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.multiply(1e-4, p1, 3.0, A, B)
    mw.multiply(1e-4, p2, [(3.0, A), (1.0, B)])
    assert p1.square_norm == p2.square_norm


@pytest.mark.parametrize("basis,order", [(mw.INTERPOLATING, 5), (mw.LEGENDRE, 7)])
def test_multiply_max_norms_gpu_vs_oracle(gpu, basis, order):
    # multiply(..., useMaxNorms = true): the grid from the two inputs' max norms
    # (MultiplicationAdaptor.h:45-65); a different grid from the wavelet adaptor's
    mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
    A = project(mra, 1e-5, gaussian_sum(51, 3, (0.5, 20.0), (-1.5, 1.5)))
    B = project(mra, 1e-5, gaussian_sum(52, 2, (1.0, 10.0), (-1.0, 1.0)))
    terms = [(2.0, A), (1.0, B)]
    g = mw.FunctionTree(mra)
    st = mw.multiply(1e-5, g, terms, use_max_norms=True)
    ref = oracle.combine(1, 1e-5, mw.FunctionTree(mra), terms, use_max_norms=True)
    plain = oracle.combine(1, 1e-5, mw.FunctionTree(mra), terms)
    assert ref["n_nodes"] != plain["n_nodes"]
    gx = g.export()
    same, perm = match(gx, ref)
    assert same, "max-norm grid differs from the oracle"
    mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
    assert mx <= 1e-12 and l2 <= 1e-12, (mx, l2)
    assert st["iterations"] == ref["iterations"]
    # the max-norm adaptor never refines below both inputs' grids
    depth = lambda x: int(x["idx"][:, 0].max())
    assert depth(gx) <= max(depth(A.export()), depth(B.export()))
    with pytest.raises(RuntimeError, match="two functions"):
        mw.multiply(1e-5, mw.FunctionTree(mra), [(1.0, A), (1.0, B), (1.0, A)], use_max_norms=True)
