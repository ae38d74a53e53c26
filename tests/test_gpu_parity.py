"""GPU parity: the CUDA path (through the C-ABI) against the CPU oracle on the
same seeded inputs.  FP64 form: identical output topology and node-term
counts, coefficients within 1e-11 of the largest coefficient (only the FP64
summation order differs).  Mixed form: global relative L2 error <= 1e-5."""
import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, project, rel_errors, unit_gaussian

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
MIXED_TOL = 1e-5


def run_pair(prec, mra, oper, f, out_gpu, out_ref, max_iter=-1, precision=mw.FP64):
    st = mw.apply(prec, out_gpu, oper, f, max_iter=max_iter, precision=precision)
    ref = oracle.apply(prec, out_ref, oper, f, max_iter=max_iter)
    return st, out_gpu.export(), ref


def check_fp64(st, gx, ref):
    same, perm = match(gx, ref)
    assert same, "output topology differs from the oracle"
    mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
    assert mx <= FP64_TOL, mx
    assert l2 <= FP64_TOL, l2
    assert st["node_terms"] == ref["node_terms"]
    assert st["components"] == ref["components"]


def test_poisson_adaptive_interpolating_k5(gpu):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    f = project(mra, 1e-3, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    st, gx, ref = run_pair(1e-3, mra, P, f, mw.FunctionTree(mra), mw.FunctionTree(mra))
    check_fp64(st, gx, ref)


def test_poisson_fixed_grid_legendre(gpu):
    mra = mw.MRA(box=(-32, 32), order=5, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = project(mra, 1e-4, gaussian_sum(7, 4, (1.0, 30.0), (-3.0, 3.0)))
    # reference grid: the oracle's adaptive output; then apply with maxIter = 0 on a copy
    grid = oracle.to_tree(oracle.apply(1e-4, mw.FunctionTree(mra), P, f, count_terms=False), mra)
    g1 = mw.FunctionTree(mra)
    g2 = mw.FunctionTree(mra)
    mw.copy_grid(g1, grid)
    mw.copy_grid(g2, grid)
    st, gx, ref = run_pair(1e-4, mra, P, f, g1, g2, max_iter=0)
    check_fp64(st, gx, ref)
    assert st["iterations"] == 1


def test_helmholtz_adaptive(gpu):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.LEGENDRE)
    H = mw.HelmholtzOperator(mra, 1.0, 1e-3)
    f = project(mra, 1e-3, gaussian_sum(3, 3, (2.0, 20.0), (-2.0, 2.0)))
    st, gx, ref = run_pair(1e-3, mra, H, f, mw.FunctionTree(mra), mw.FunctionTree(mra))
    check_fp64(st, gx, ref)


def test_world_border_and_uneven_box(gpu):
    # the reference test world: scale 1, corner (-1, 0, 1), 1 x 2 x 3 root boxes
    mra = mw.MRA(order=4, basis=mw.INTERPOLATING, scale=1, corner=(-1, 0, 1), nbox=(1, 2, 3), sf=1.0)
    P = mw.PoissonOperator(mra, 1e-3)
    f = project(mra, 1e-3, unit_gaussian(300.0, (-0.45, 0.05, 1.9)))  # close to three world faces
    st, gx, ref = run_pair(1e-3, mra, P, f, mw.FunctionTree(mra), mw.FunctionTree(mra))
    check_fp64(st, gx, ref)


def test_mixed_precision_error(gpu):
    mra = mw.MRA(box=(-32, 32), order=5, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = project(mra, 1e-4, gaussian_sum(11, 4, (1.0, 30.0), (-3.0, 3.0)))
    grid = oracle.to_tree(oracle.apply(1e-4, mw.FunctionTree(mra), P, f, count_terms=False), mra)
    g1, g2 = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.copy_grid(g1, grid)
    mw.copy_grid(g2, grid)
    st, gx, ref = run_pair(1e-4, mra, P, f, g1, g2, max_iter=0, precision=mw.MIXED)
    same, perm = match(gx, ref)
    assert same
    mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
    assert l2 <= MIXED_TOL, l2
    assert st["node_terms"] == ref["node_terms"]


def test_mixed_adaptive_interpolating_k5(gpu):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    f = project(mra, 1e-3, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    st, gx, ref = run_pair(1e-3, mra, P, f, mw.FunctionTree(mra), mw.FunctionTree(mra), precision=mw.MIXED)
    same, perm = match(gx, ref)
    assert same, "mixed-form adaptive topology differs from the oracle"
    # the screening decisions of the mixed form (FP32 estimate, FP64 near the
    # threshold) are the reference's: the same node-term and component counts
    assert st["node_terms"] == ref["node_terms"] and st["components"] == ref["components"]
    mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
    assert l2 <= MIXED_TOL, l2


def test_mixed_k7_fixed_grid(gpu):
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = project(mra, 1e-4, gaussian_sum(5, 3, (1.0, 30.0), (-3.0, 3.0)))
    grid = mw.FunctionTree(mra)
    mw.apply(1e-4, grid, P, f, precision=mw.FP64)
    g1, g2 = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.copy_grid(g1, grid)
    mw.copy_grid(g2, grid)
    s1 = mw.apply(1e-4, g1, P, f, max_iter=0, precision=mw.MIXED)
    s2 = mw.apply(1e-4, g2, P, f, max_iter=0, precision=mw.FP64)
    a, b = g1.export()["coefs"], g2.export()["coefs"]
    assert s1["node_terms"] == s2["node_terms"]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= MIXED_TOL


def test_mixed_orders_in_sequence(gpu):
    # one context serves levels of different orders one after the other; its
    # work buffers must follow the larger coefficient blocks
    for order in (4, 7, 5, 9):
        mra = mw.MRA(box=(-20, 20), order=order, basis=mw.LEGENDRE)
        P = mw.PoissonOperator(mra, 1e-3)
        f = project(mra, 1e-3, gaussian_sum(order, 2, (2.0, 20.0), (-1.0, 1.0)))
        g1, g2 = mw.FunctionTree(mra), mw.FunctionTree(mra)
        s1 = mw.apply(1e-3, g1, P, f, precision=mw.FP64)
        mw.copy_grid(g2, g1)
        s2 = mw.apply(1e-3, g2, P, f, max_iter=0, precision=mw.MIXED)
        g3 = mw.FunctionTree(mra)
        mw.copy_grid(g3, g1)
        mw.apply(1e-3, g3, P, f, max_iter=0, precision=mw.FP64)
        a, b = g2.export()["coefs"], g3.export()["coefs"]
        assert np.isfinite(a).all()
        assert np.linalg.norm(a - b) / np.linalg.norm(b) <= MIXED_TOL, order


def test_helmholtz_k9_mixed_vs_fp64_and_oracle(gpu):
    # Helmholtz (mu = 1), Legendre k=9: the mixed form against the FP64 form
    # (global and per-node error) and the FP64 form against the oracle
    mra = mw.MRA(box=(-32, 32), order=9, basis=mw.LEGENDRE)
    H = mw.HelmholtzOperator(mra, 1.0, 1e-4)
    f = project(mra, 1e-4, gaussian_sum(31, 3, (0.5, 20.0), (-2.0, 2.0)))
    g64 = mw.FunctionTree(mra)
    st = mw.apply(1e-4, g64, H, f, precision=mw.FP64)
    ref = oracle.apply(1e-4, mw.FunctionTree(mra), H, f)
    check_fp64(st, g64.export(), ref)
    gm = mw.FunctionTree(mra)
    mw.copy_grid(gm, g64)
    mw.apply(1e-4, gm, H, f, max_iter=0, precision=mw.MIXED)
    g2 = mw.FunctionTree(mra)
    mw.copy_grid(g2, g64)
    mw.apply(1e-4, g2, H, f, max_iter=0, precision=mw.FP64)
    a, b = gm.export(), g2.export()
    assert np.linalg.norm(a["coefs"] - b["coefs"]) / np.linalg.norm(b["coefs"]) <= MIXED_TOL
    # per node, relative to the largest node norm
    per_node = np.linalg.norm(a["coefs"] - b["coefs"], axis=1) / np.linalg.norm(b["coefs"], axis=1).max()
    assert per_node.max() <= MIXED_TOL


@pytest.mark.parametrize("adaptive", [False, True])
def test_tcgen05_contraction_k7(gpu, monkeypatch, adaptive):
    # the opt-in tcgen05 contraction (order 7, MWGPU_TC) against the FP64 form:
    # same node-term count, relative L2 error <= 1e-5 per apply; on the fixed
    # grid every item is a block-schedule item (tensor-core chunks only), the
    # adaptive apply mixes in screened items (CUDA-core chunks)
    mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-4)
    f = project(mra, 1e-4, gaussian_sum(11, 4, (1.0, 50.0), (-3.0, 3.0)))
    grid = mw.FunctionTree(mra)
    s0 = mw.apply(1e-4, grid, P, f, precision=mw.FP64)
    monkeypatch.setenv("MWGPU_TC", "1")
    g1, g2 = mw.FunctionTree(mra), mw.FunctionTree(mra)
    if adaptive:
        s1 = mw.apply(1e-4, g1, P, f, precision=mw.MIXED)
        same, perm = match(g1.export(), grid.export())
        assert same, "topology differs from the FP64 form"
        a, b = g1.export()["coefs"], grid.export()["coefs"][perm]
        assert s1["node_terms"] == s0["node_terms"]
    else:
        mw.copy_grid(g1, grid)
        mw.copy_grid(g2, grid)
        s1 = mw.apply(1e-4, g1, P, f, max_iter=0, precision=mw.MIXED)
        monkeypatch.delenv("MWGPU_TC")
        s2 = mw.apply(1e-4, g2, P, f, max_iter=0, precision=mw.FP64)
        a, b = g1.export()["coefs"], g2.export()["coefs"]
        assert s1["node_terms"] == s2["node_terms"]
    assert np.isfinite(a).all()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= MIXED_TOL
