"""Multiwavelet filter and cross-correlation tables.

The product ships tables computed from first principles
(mrcpp_gb300/data/gen_mwtables.py).  They are pinned against the reference's
own shipped tables (golden fixture tests/golden/mwfilters_ref.npz, made by
tests/golden/make_golden.py from share/mwfilters) and against the filter
orthonormality test of the reference (tests/core/mw_filter.cpp:36-61).
"""
import os

import numpy as np
import pytest

from mrcpp_gb300 import tables

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mwfilters_ref.npz")


@pytest.fixture(scope="module")
def tab():
    return tables.load()


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _orders(gold, prefix):
    return sorted({int(k.split("_")[-1]) for k in gold.files if k.startswith(prefix)})


@pytest.mark.parametrize("t,typ", [("L", 0), ("I", 1)])
def test_scaling_filters_match_reference(tab, gold, t, typ):
    for k in _orders(gold, t + "_H0"):
        np.testing.assert_allclose(tab[(tables.H0, typ, k)], gold["%s_H0_%d" % (t, k)], rtol=0, atol=1e-15)


@pytest.mark.parametrize("t,typ", [("L", 0), ("I", 1)])
def test_wavelet_filters_match_reference_up_to_sign(tab, gold, t, typ):
    # each wavelet is unique up to sign (Alpert's vanishing-moment conditions)
    for k in _orders(gold, t + "_G0"):
        a, b = tab[(tables.G0, typ, k)], gold["%s_G0_%d" % (t, k)]
        s = np.sign((a * b).sum(axis=1))
        assert np.all(s != 0)
        np.testing.assert_allclose(a, s[:, None] * b, rtol=0, atol=1e-15)


@pytest.mark.parametrize("t,typ", [("L", 0), ("I", 1)])
def test_cross_correlation_matches_reference(tab, gold, t, typ):
    for k in _orders(gold, t + "_c_left"):
        for kind, side in ((tables.CLEFT, "left"), (tables.CRIGHT, "right")):
            ref = gold["%s_c_%s_%d" % (t, side, k)]
            np.testing.assert_allclose(tab[(kind, typ, k)], ref, rtol=0, atol=1e-15)


def _full_filter(H0, G0, typ):
    K = H0.shape[0]
    i, j = np.meshgrid(np.arange(K), np.arange(K), indexing="ij")
    if typ == 1:
        G1 = (-1.0) ** (i + K) * G0[:, ::-1]
        H1 = H0[::-1, ::-1]
    else:
        G1 = (-1.0) ** (i + j + K) * G0
        H1 = (-1.0) ** (i + j) * H0
    return np.block([[G0, G1], [H0, H1]])


@pytest.mark.parametrize("typ", [0, 1])
def test_filter_orthonormality(tab, typ):
    # the two-scale filter is orthogonal for every shipped order (reference: k <= 40)
    for k in range(0, 26):
        F = _full_filter(tab[(tables.H0, typ, k)], tab[(tables.G0, typ, k)], typ)
        np.testing.assert_allclose(F @ F.T, np.eye(F.shape[0]), atol=1e-13)
        np.testing.assert_allclose(F.T @ F, np.eye(F.shape[0]), atol=1e-13)


def test_alpert_vanishing_moments(tab):
    # psi_i is orthogonal to all polynomials of degree < K + i on [0, 1]
    from numpy.polynomial import legendre as npl

    for k in (1, 3, 5, 7):
        K = k + 1
        G0 = tab[(tables.G0, 0, k)]
        x, w = npl.leggauss(2 * K + 2)
        x = 0.5 * (x + 1.0)
        w = 0.5 * w

        def phi(j, t):
            c = np.zeros(j + 1)
            c[j] = 1.0
            return np.sqrt(2 * j + 1) * npl.legval(2 * t - 1, c)

        i_, j_ = np.meshgrid(np.arange(K), np.arange(K), indexing="ij")
        G1 = (-1.0) ** (i_ + j_ + K) * G0
        for i in range(K):
            for m in range(K + i):
                # integrate psi_i * P_m(2x-1) over the two halves
                left = sum(G0[i, j] * np.sqrt(2) * np.sum(0.5 * w * phi(j, x) * phi(m, 0.5 * x)) for j in range(K))
                right = sum(G1[i, j] * np.sqrt(2) * np.sum(0.5 * w * phi(j, x) * phi(m, 0.5 + 0.5 * x)) for j in range(K))
                assert abs(left + right) < 1e-13, (k, i, m)
