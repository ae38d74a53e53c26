"""Projection on the GPU (mwgpu_project_level / mwgpu_project_level_values
through the host TreeBuilder loop) against the oracle's projection and the
host mirror's (both restate project / ProjectionCalculator on the CPU):
identical grid, FP64 coefficients within 1e-12 of the largest, and the
analytic norm and integral of the projected Gaussians."""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
from cases import gaussian_sum, match, rel_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("basis,order,prec", [(mw.INTERPOLATING, 5, 1e-3), (mw.LEGENDRE, 7, 1e-5), (mw.LEGENDRE, 9, 1e-6)])
def test_project_gpu_vs_host(gpu, basis, order, prec):
    mra = mw.MRA(box=(-32, 32), order=order, basis=basis)
    gs = gaussian_sum(41, 6, (1.0, 60.0), (-3.0, 3.0))
    a, b = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.project(prec, a, gs)
    st = mw.project(prec, b, gs, device=True)
    same, perm = match(b.export(), {"idx": a.export()["idx"]})
    assert same, "grid differs from the host projection"
    mx, l2 = rel_errors(b.export()["coefs"], a.export()["coefs"][perm])
    assert mx <= 1e-12 and l2 <= 1e-12, (mx, l2)
    assert b.square_norm == pytest.approx(a.square_norm, rel=1e-12)
    assert st["out_nodes"] == a.n_nodes and st["iterations"] >= 1


def test_project_gpu_unit_gaussian_norm_and_integral(gpu):
    # a normalised Gaussian: integral 1, squared norm (beta/pi)^3 (pi/(2 beta))^(3/2)
    mra = mw.MRA(box=(-20, 20), order=6, basis=mw.LEGENDRE)
    beta = 25.0
    f = mw.FunctionTree(mra)
    mw.project(1e-6, f, [((beta / math.pi) ** 1.5, beta, (0.3, -0.2, 0.1))], device=True)
    assert f.integrate() == pytest.approx(1.0, abs=1e-7)
    exact = (beta / math.pi) ** 3 * (math.pi / (2 * beta)) ** 1.5
    assert f.square_norm == pytest.approx(exact, rel=1e-7)


def test_project_gpu_feeds_apply(gpu):
    # a device-projected input gives the same Poisson apply as a host-projected one
    mra = mw.MRA(box=(-32, 32), order=5, basis=mw.INTERPOLATING)
    gs = gaussian_sum(43, 3, (2.0, 20.0), (-1.0, 1.0))
    P = mw.PoissonOperator(mra, 1e-3)
    fa, fb = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.project(1e-3, fa, gs)
    mw.project(1e-3, fb, gs, device=True)
    ga, gb = mw.FunctionTree(mra), mw.FunctionTree(mra)
    mw.apply(1e-3, ga, P, fa)
    mw.apply(1e-3, gb, P, fb)
    same, perm = match(gb.export(), {"idx": ga.export()["idx"]})
    assert same
    mx, _ = rel_errors(gb.export()["coefs"], ga.export()["coefs"][perm])
    assert mx <= 1e-11


@pytest.mark.parametrize("basis,order", [(mw.LEGENDRE, 7), (mw.INTERPOLATING, 5)])
def test_device_projection_vs_oracle(gpu, basis, order):
    # project(prec, tree, func) with the nodes on the GPU: a Slater function
    # evaluated on the host per level (mwgpu_project_level_values) and a
    # Gaussian sum evaluated on the device (mwgpu_project_level), both against
    # the oracle's projection: the same grid, coefficients within 1e-12
    import oracle
    from cases import gaussian_sum, match, rel_errors

    mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
    slater = lambda r: np.exp(-np.linalg.norm(r, axis=1)) / np.sqrt(np.pi)
    gs = gaussian_sum(31, 3, (1.0, 40.0), (-2.0, 2.0))

    def gsum(r):
        v = np.zeros(len(r))
        for c, a, R in gs:
            v += c * np.exp(-a * ((r - np.asarray(R)) ** 2).sum(axis=1))
        return v

    for f, dev in ((slater, lambda t: mw.project(1e-5, t, slater, device=True)),
                   (gsum, lambda t: mw.project(1e-5, t, gs, grid=False, device=True))):
        ref = oracle.project(1e-5, mw.FunctionTree(mra), f)
        t = mw.FunctionTree(mra)
        st = dev(t)
        tx = t.export()
        same, perm = match(tx, ref)
        assert same, "grid differs from the oracle's"
        mx, l2 = rel_errors(tx["coefs"], ref["coefs"][perm])
        assert mx <= 1e-12 and l2 <= 1e-12, (mx, l2)
        assert st["iterations"] == ref["iterations"]
