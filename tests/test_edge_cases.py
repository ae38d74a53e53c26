"""Edge cases of the apply path.

* A zero input (a projected Gaussian with coefficient 0: a refined grid whose
  coefficients are all zero): every component fails the MachineZero screen
  (ConvolutionCalculator.cpp:258), the work lists are empty, the output is
  zero on the roots and nothing is refined (split_check with a zero norm).
* Inputs refined many levels below the root scale (unit Gaussians of exponent
  1e6 in [-20, 20]^3 and 1e12 in [-32, 32]^3, output depths 13 and 23):
  GenNodes and operator bands at deep levels; at depth 23 the translations
  need more than 19 bits per direction (2 root boxes x 2^23).
* A batch that mixes zero and non-zero inputs (empty per-tree segments of a
  batched level).

CPU: the oracle.  GPU: the CUDA path against the oracle (FP64: coefficients to
1e-11 of the largest, identical counts; mixed: relative L2 error <= 1e-5).
"""
import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import match, rel_errors, unit_gaussian

PREC = 1e-3


def zero_input(mra):
    f = mw.FunctionTree(mra)
    mw.project(PREC, f, [(0.0, 50.0, (0.1, 0.2, 0.3))])
    return f


def deep_input(mra, beta=1e6):
    f = mw.FunctionTree(mra)
    mw.project(PREC, f, unit_gaussian(beta, (0.013, -0.021, 0.007)))
    return f


DEEP = [((-20, 20), 1e6, 10), ((-32, 32), 1e12, 21)]  # box, exponent, least output depth


def depths(flat):
    return np.unique(flat["idx"][:, 0])


def test_oracle_zero_input():
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, PREC)
    f = zero_input(mra)
    assert f.n_nodes > 8 and f.square_norm == 0.0
    ref = oracle.apply(PREC, mw.FunctionTree(mra), P, f)
    assert ref["node_terms"] == 0 and ref["components"] == 0
    assert ref["n_nodes"] == 8  # the roots: a zero function is not refined
    assert not np.any(ref["coefs"])


@pytest.mark.parametrize("box, beta, min_depth", DEEP)
def test_oracle_deep_input_levels(box, beta, min_depth):
    mra = mw.MRA(box=box, order=5, basis=mw.INTERPOLATING)
    f = deep_input(mra, beta)
    assert depths(f.export()).max() - mra.root_scale >= min_depth + 2


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [mw.FP64, mw.MIXED])
def test_gpu_zero_input(gpu, precision):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, PREC)
    f = zero_input(mra)
    g = mw.FunctionTree(mra)
    st = mw.apply(PREC, g, P, f, precision=precision)
    gx = g.export()
    ref = oracle.apply(PREC, mw.FunctionTree(mra), P, f)
    same, _ = match(gx, ref)
    assert same
    assert st["node_terms"] == 0
    assert not np.any(gx["coefs"])
    assert g.square_norm == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [mw.FP64, mw.MIXED])
@pytest.mark.parametrize("box, beta, min_depth", DEEP)
def test_gpu_deep_input(gpu, precision, box, beta, min_depth):
    mra = mw.MRA(box=box, order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, PREC)
    f = deep_input(mra, beta)
    g = mw.FunctionTree(mra)
    st = mw.apply(PREC, g, P, f, precision=precision)
    gx = g.export()
    ref = oracle.apply(PREC, mw.FunctionTree(mra), P, f)
    same, perm = match(gx, ref)
    assert same, "output topology differs from the oracle"
    mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
    if precision == mw.FP64:
        assert mx <= 1e-11 and l2 <= 1e-11, (mx, l2)
        assert st["node_terms"] == ref["node_terms"]
        assert st["components"] == ref["components"]
    else:
        assert l2 <= 1e-5, l2
    assert depths(gx).max() - mra.root_scale >= min_depth


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [mw.FP64, mw.MIXED])
def test_gpu_batch_with_zero_members(gpu, precision):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, PREC)
    fs = [zero_input(mra), mw.FunctionTree(mra), zero_input(mra)]
    mw.project(PREC, fs[1], unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    outs = [mw.FunctionTree(mra) for _ in fs]
    mw.apply_batch(PREC, outs, P, fs, precision=precision)
    for out, f in zip(outs, fs):
        gx = out.export()
        ref = oracle.apply(PREC, mw.FunctionTree(mra), P, f)
        same, perm = match(gx, ref)
        assert same
        if not np.any(ref["coefs"]):
            assert not np.any(gx["coefs"])
            continue
        mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
        assert l2 <= (1e-11 if precision == mw.FP64 else 1e-5), l2
