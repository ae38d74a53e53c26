"""Operator blocks and norms of the product's operator construction, recomputed
from their definition with nothing of the product but the wavelet sign
convention (CPU).

For a kernel term c exp(-alpha x^2) (coefficient c^(1/3) per dimension,
ConvolutionOperator.cpp:84-86), scale n, unit length h = sf 2^-n and
translation l, the four components of the operator node are

    O_ab(l)[p, q] = h int int f^a_p(u) k(h (u - v - l)) f^b_q(v) du dv,

f^0 = the Legendre scaling functions sqrt(2j+1) P_j(2u-1) on [0, 1], f^1 = the
multiwavelets made from them by the reference's shipped two-scale filters
(tests/golden/mwfilters_ref.npz, G1 by the symmetry of MWFilter.cpp:240).
This is what ConvolutionOperator.cpp:78-108 and CrossCorrelationCalculator.cpp
:36-96 compute through a projected kernel and cross-correlation tables; here
the double integral is the cross-correlation C_pq(tau) = int f_p(u) f_q(u-tau)
du (exact Gauss-Legendre per polynomial piece) integrated against the
Gaussian with panels graded toward its peak.  The product exports the block
of translation l as O(-l) in this convention, column-major.

Component norms: OperatorNode::calcComponentNorm (OperatorNode.cpp:56-80):
math_utils::matrix_norm_2 (math_utils.cpp:60-62) is Eigen's lpNorm<2>(), the
coefficient-wise l2 norm of the block, behind the vector and 1-inf norm
thresholds max(MachinePrec, prec / (8 2^depth)).
"""
import os

import numpy as np
import pytest
from numpy.polynomial import legendre as npleg

import mrcpp_gb300 as mw
from mrcpp_gb300 import tables

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "mwfilters_ref.npz"))
GX, GW = npleg.leggauss(24)
MACHINE_PREC = 1e-15


def phi(K, t):
    out = np.empty((K,) + t.shape)
    for j in range(K):
        c = np.zeros(j + 1)
        c[j] = 1.0
        out[j] = np.sqrt(2 * j + 1) * npleg.legval(2 * t - 1, c)
    return out


def wavelets(K, t, G0, G1):
    lo = t < 0.5
    a = np.sqrt(2) * np.tensordot(G0, phi(K, 2 * t), axes=(1, 0))
    b = np.sqrt(2) * np.tensordot(G1, phi(K, 2 * t - 1), axes=(1, 0))
    return np.where(lo, a, b)


def correlations(K, tau, G0, G1):
    """C[ka, kb][p, q, i] = int f^ka_p(u) f^kb_q(u - tau_i) du, all i at once:
    the overlap [max(0,tau), min(1,1+tau)] cut at the wavelets' midpoints."""
    lo, hi = np.maximum(0.0, tau), np.minimum(1.0, 1.0 + tau)
    b1 = np.clip(np.minimum(0.5, tau + 0.5), lo, hi)
    b2 = np.clip(np.maximum(0.5, tau + 0.5), lo, hi)
    C = np.zeros((2, 2, K, K, len(tau)))
    for a, b in ((lo, b1), (b1, b2), (b2, hi)):
        u = 0.5 * (b - a)[:, None] * GX + 0.5 * (a + b)[:, None]
        w = 0.5 * (b - a)[:, None] * GW
        fu = (phi(K, u), wavelets(K, u, G0, G1))
        fv = (phi(K, u - tau[:, None]), wavelets(K, u - tau[:, None], G0, G1))
        for ka in range(2):
            for kb in range(2):
                C[ka, kb] += np.einsum("pij,ij,qij->pqi", fu[ka], w, fv[kb])
    return C


def blocks(K, alpha, coef, h, l, G0, G1):
    """O_ab(l) for the four components (index ka + 2 kb)."""
    sig = 1.0 / (h * np.sqrt(2.0 * alpha))
    bps = {-1.0, -0.5, 0.0, 0.5, 1.0}
    if -1 < l < 1:
        bps.add(float(l))
    w = sig
    while w < 2.0:
        for x in (l - w, l + w):
            if -1 < x < 1:
                bps.add(x)
        w *= 2.0
    bps = sorted(bps)
    a, b = np.array(bps[:-1]), np.array(bps[1:])
    tau = (0.5 * (b - a)[:, None] * GX + 0.5 * (a + b)[:, None]).ravel()
    wt = (0.5 * (b - a)[:, None] * GW).ravel()
    kv = coef * np.exp(-alpha * (h * (tau - l)) ** 2) * wt
    C = correlations(K, tau, G0, G1)
    return [h * (C[c & 1, c >> 1] * kv).sum(axis=2) for c in range(4)]


def rows(ex):
    """(term, depth, offset of l = -L, L) of every row of the node cache."""
    out, off, r = [], 0, 0
    for t, nd in enumerate(ex["depth"]):
        for d in range(nd):
            L = int(ex["max_transl"][r])
            out.append((t, d, off, L))
            off += 2 * L + 1
            r += 1
    return out


@pytest.mark.parametrize("order", [5, 7])
def test_blocks_from_the_definition(order):
    K = order + 1
    mra = mw.MRA(box=(-32, 32), order=order, basis=mw.LEGENDRE)
    d = mra.desc()
    P = mw.PoissonOperator(mra, 1e-5)
    ex = P.export()
    G0 = GOLDEN["L_G0_%d" % order]
    G1 = np.array([[(-1.0) ** (i + j + K) * G0[i, j] for j in range(K)] for i in range(K)])
    # the product's multiwavelets may differ from the shipped ones in sign only
    sgn = np.sign((tables.load()[(tables.G0, 0, order)] * G0).sum(axis=1))
    nodes = ex["blocks"].reshape(-1, 4, K, K)
    T = P.n_terms
    terms = {0, T // 3, (2 * T) // 3, T - 1}
    checked = 0
    for t, dep, off, L in rows(ex):
        if t not in terms or dep not in (0, int(ex["depth"][t]) - 1):
            continue
        h = d.sf * 2.0 ** (-(d.root_scale + dep))
        a, c = ex["kernel_exp"][t], ex["kernel_coef"][t]
        c3 = np.copysign(abs(c) ** (1.0 / 3.0), c)
        scale = np.abs(nodes[off:off + 2 * L + 1]).max()
        for l in sorted({0, 1, -1, L}):
            if abs(l) > L:
                continue
            q = blocks(K, a, c3, h, -l, G0, G1)
            for comp in range(4):
                s = np.outer(sgn if comp & 1 else np.ones(K), sgn if comp >> 1 else np.ones(K))
                got = nodes[off + l + L][comp].T
                err = np.abs(got - q[comp] * s).max() / scale
                assert err <= 1e-10, (order, t, dep, l, comp, err)
                checked += 1
    assert checked >= 40


def test_component_norms():
    order, K = 7, 8
    mra = mw.MRA(box=(-32, 32), order=order, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, 1e-5)
    ex = P.export()
    nodes = ex["blocks"].reshape(-1, 4, K, K)
    norms = ex["norms"].reshape(-1, 4)
    prec = 1e-5
    n_pos = 0
    for t, dep, off, L in rows(ex):
        thrs = max(MACHINE_PREC, prec / (8.0 * (1 << dep)))
        for j in range(off, off + 2 * L + 1):
            for comp in range(4):
                m = nodes[j][comp].T
                two = vec = np.sqrt((m * m).sum())
                one, inf = np.abs(m).sum(axis=0).max(), np.abs(m).sum(axis=1).max()
                want = two if (vec > thrs and np.sqrt(inf * one) > thrs and two > thrs) else 0.0
                # at the thresholds themselves either answer is right
                if min(abs(vec - thrs), abs(np.sqrt(inf * one) - thrs), abs(two - thrs)) < 1e-9 * thrs:
                    continue
                assert norms[j][comp] == pytest.approx(want, rel=1e-13, abs=0.0), (t, dep, j - off - L, comp)
                n_pos += want > 0
    assert n_pos > 1000
