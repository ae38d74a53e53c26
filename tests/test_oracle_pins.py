"""Pins of the CPU oracle and of the operator construction against the
reference's own known-answer tests (CPU only).

  Poisson kernel      tests/operators/poisson_operator.cpp:47-71 (26 terms, 2 eps accuracy)
  Helmholtz kernel    tests/operators/helmholtz_operator.cpp:48-73 (33 terms, 2 eps accuracy)
  band widths         tests/operators/poisson_operator.cpp:100-121 (monotone in the precision)
  Coulomb energy      tests/operators/poisson_operator.cpp:129-154 (relative 1e-3, analytic Boys F0)
  potentials          the analytic erf(sqrt(b) r)/r (Poisson) and Yukawa (Helmholtz) potentials
                      of a normalised Gaussian
"""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
import oracle
from cases import project, unit_gaussian


def test_poisson_kernel_known_answer():
    eps, r_min, r_max = 1e-4, 1e-3, 1.0
    ex, co = mw.poisson_kernel(eps, r_min, r_max)
    assert len(ex) == 26
    x = r_min
    while x < r_max:
        v = float(np.sum(co * np.exp(-ex * x * x)))
        assert v == pytest.approx(1.0 / x, rel=2 * eps)
        x *= 1.5


def test_helmholtz_kernel_known_answer():
    mu, eps, r_min, r_max = 0.01, 1e-4, 1e-3, 1.0
    ex, co = mw.helmholtz_kernel(mu, eps, r_min, r_max)
    assert len(ex) == 33
    x = r_min
    while x < r_max:
        v = float(np.sum(co * np.exp(-ex * x * x)))
        assert v == pytest.approx(math.exp(-mu * x) / x, rel=2 * eps)
        x *= 1.5


@pytest.mark.parametrize("box,prec,n_poisson,n_helm", [((-20, 20), 1e-3, 49, 38), ((-20, 20), 1e-5, 79, 62), ((-32, 32), 1e-6, 96, 75)])
def test_operator_term_counts(box, prec, n_poisson, n_helm):
    # PoissonOperator/HelmholtzOperator use k_prec = prec/10, r_min = sqrt(k_prec 2^-maxScale), r_max = box diagonal
    mra = mw.MRA(box=box, order=5, basis=mw.INTERPOLATING)
    k_prec = prec / 10
    r_min = math.sqrt(k_prec * 2.0 ** (-mra.max_scale))
    r_max = math.sqrt(3.0) * (box[1] - box[0])
    assert len(mw.poisson_kernel(k_prec, r_min, r_max)[0]) == n_poisson
    assert len(mw.helmholtz_kernel(1.0, k_prec, r_min, r_max)[0]) == n_helm


def _bandwidths(ex, prec):
    """OperatorTree::calcBandWidth on the exported node caches: widths[term][depth]."""
    depth, mt, norms = ex["depth"], ex["max_transl"], ex["norms"].reshape(-1, 4)
    out, node, row = [], 0, 0
    for t in range(len(depth)):
        w = []
        for d in range(depth[t]):
            L = mt[row + d]
            thrs = max(1e-15, prec / (8.0 * 2 ** d))
            best, l = -1, 0
            while True:
                done = True
                for c in range(4):
                    if norms[node + l + L, c] > thrs:
                        best, done = l, False
                l += 1
                if l > L or done:
                    break
            w.append(best)
            node += 2 * L + 1
        row += depth[t]
        out.append(w)
    return out


def test_bandwidth_monotone_in_precision():
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    ex = P.export()
    b1, b2, b3 = _bandwidths(ex, 1.0), _bandwidths(ex, 1e-3), _bandwidths(ex, -1 if False else 1e-3 / 10)
    for t in range(P.n_terms):
        for d in range(len(b1[t])):
            assert b1[t][d] <= b2[t][d] <= b3[t][d]


def test_coulomb_energy_known_answer():
    # the reference's test world: scale 1, corner (-1, 0, 1), 1 x 2 x 3 boxes, interpolating k=5
    mra = mw.MRA(order=5, basis=mw.INTERPOLATING, scale=1, corner=(-1, 0, 1), nbox=(1, 2, 3), sf=1.0)
    P = mw.PoissonOperator(mra, 1e-4)
    beta = 1e4
    f = mw.FunctionTree(mra)
    mw.project(1e-4, f, unit_gaussian(beta, (-0.2, 0.5, 1.0)), grid=False)
    g = oracle.to_tree(oracle.apply(1e-3, mw.FunctionTree(mra), P, f, count_terms=False), mra)
    E = mw.dot(g, f)
    E_ana = math.sqrt(2 * beta / math.pi)  # GaussFunc::calcCoulombEnergy of a unit Gaussian with itself
    assert E == pytest.approx(E_ana, rel=1e-3)


def test_poisson_potential_erf():
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-3)
    beta, c = 10.0, np.array([0.1, 0.2, -0.3])
    f = project(mra, 1e-3, unit_gaussian(beta, c))
    g = oracle.to_tree(oracle.apply(1e-3, mw.FunctionTree(mra), P, f, count_terms=False), mra)
    rng = np.random.default_rng(1)
    errs = []
    for _ in range(60):
        r = float(np.exp(rng.uniform(np.log(0.05), np.log(8.0))))
        u = rng.normal(size=3)
        x = c + r * u / np.linalg.norm(u)
        errs.append((g.evalf(x) - math.erf(math.sqrt(beta) * r) / r) / (math.erf(math.sqrt(beta) * r) / r))
    # prec bounds the L2 error relative to the norm of the whole potential; pointwise
    # relative errors at 1e-3 stay within 1e-2 over the sampled shell
    assert np.sqrt(np.mean(np.square(errs))) < 1e-2
    assert mw.dot(g, f) == pytest.approx(math.sqrt(2 * beta / math.pi), rel=1e-3)


def yukawa_gaussian(r, beta, mu):
    """int exp(-mu|x-y|)/|x-y| rho(y) dy for rho = (beta/pi)^1.5 exp(-beta |y|^2)."""
    a = mu / (2.0 * math.sqrt(beta))
    sb = math.sqrt(beta)
    pre = math.exp(mu * mu / (4.0 * beta)) / (2.0 * r)
    return pre * (math.exp(-mu * r) * math.erfc(a - sb * r) - math.exp(mu * r) * math.erfc(a + sb * r))


def test_helmholtz_potential_yukawa():
    mu, beta = 1.0, 10.0
    # the closed form reduces to the Coulomb potential for mu -> 0
    assert yukawa_gaussian(0.7, beta, 1e-9) == pytest.approx(math.erf(math.sqrt(beta) * 0.7) / 0.7, rel=1e-7)
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.LEGENDRE)
    H = mw.HelmholtzOperator(mra, mu, 1e-4)
    c = np.array([0.3, -0.1, 0.2])
    f = project(mra, 1e-4, unit_gaussian(beta, c))
    g = oracle.to_tree(oracle.apply(1e-4, mw.FunctionTree(mra), H, f, count_terms=False), mra)
    rng = np.random.default_rng(2)
    errs = []
    for _ in range(40):
        r = float(np.exp(rng.uniform(np.log(0.05), np.log(4.0))))
        u = rng.normal(size=3)
        x = c + r * u / np.linalg.norm(u)
        va = yukawa_gaussian(r, beta, mu)
        errs.append((g.evalf(x) - va) / va)
    assert np.sqrt(np.mean(np.square(errs))) < 1e-3
