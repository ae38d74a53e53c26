"""The FP64 form's two schedules (k_contract<double>): the block schedule (sums
over the input bit before each next 1D step, the s->s product at depth > 0
kept out exactly) and the per-component schedule (MWGPU_FP64_COMPONENTS=1),
both against the oracle: identical topology, node-term and component counts,
coefficients within 1e-11 of the largest; and against each other within
1e-13 (only the summation order differs).
"""
import os

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import gaussian_sum, match, project, rel_errors, unit_gaussian

pytestmark = pytest.mark.gpu


def run(prec, mra, oper, f, components, grid=None):
    if components:
        os.environ["MWGPU_FP64_COMPONENTS"] = "1"
    try:
        g = mw.FunctionTree(mra)
        if grid is not None:
            mw.copy_grid(g, grid)
            st = mw.apply(prec, g, oper, f, max_iter=0, precision=mw.FP64)
        else:
            st = mw.apply(prec, g, oper, f, precision=mw.FP64)
    finally:
        os.environ.pop("MWGPU_FP64_COMPONENTS", None)
    return g, st


@pytest.mark.parametrize("case", ["poisson_k5", "helmholtz_k9", "poisson_k7_screened"])
def test_block_and_component_schedules(gpu, case):
    if case == "poisson_k5":
        mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
        prec, oper = 1e-3, None
        oper = mw.PoissonOperator(mra, prec)
        f = project(mra, prec, unit_gaussian(10.0, (0.1, 0.2, -0.3)))
    elif case == "helmholtz_k9":
        mra = mw.MRA(box=(-32, 32), order=9, basis=mw.LEGENDRE)
        prec = 1e-4
        oper = mw.HelmholtzOperator(mra, 1.0, prec)
        f = project(mra, prec, gaussian_sum(7, 3, (1.0, 50.0), (-4.0, 4.0)))
    else:
        # adaptive k = 7: levels after the first screen by norm, so items take
        # both schedules within one level
        mra = mw.MRA(box=(-32, 32), order=7, basis=mw.LEGENDRE)
        prec = 1e-4
        oper = mw.PoissonOperator(mra, prec)
        f = project(mra, prec, gaussian_sum(2026, 6, (1.0, 100.0), (-5.0, 5.0)))
    ref = oracle.apply(prec, mw.FunctionTree(mra), oper, f)
    out = {}
    for comp in (False, True):
        g, st = run(prec, mra, oper, f, comp)
        gx = g.export()
        same, perm = match(gx, ref)
        assert same, (case, comp)
        assert st["node_terms"] == ref["node_terms"] and st["components"] == ref["components"], (case, comp)
        mx, l2 = rel_errors(gx["coefs"], ref["coefs"][perm])
        assert mx <= 1e-11 and l2 <= 1e-11, (case, comp, mx, l2)
        out[comp] = gx["coefs"]
    d = np.abs(out[False] - out[True]).max() / np.abs(out[True]).max()
    assert d <= 1e-13, (case, d)


def test_fp64_pipe_rates(gpu):
    # the FP64 form runs on DFMA: measured, DMMA (mma.sync m8n8k4 f64) peaks
    # lower on this GPU (1.26 against 1.10 TFLOP/s when written)
    import ctypes as C

    L = mw.lib()
    ctx = C.c_void_p()
    assert L.mwgpu_init(C.byref(ctx), C.byref(mw.MwgpuConfig())) == 0
    try:
        a, b = C.c_double(), C.c_double()
        assert L.mwgpu_fp64_pipe_rates(ctx, C.byref(a), C.byref(b)) == 0
        assert a.value > 0.1 and b.value > 0.1
        assert a.value >= 0.95 * b.value, (a.value, b.value)
    finally:
        L.mwgpu_destroy(ctx)
