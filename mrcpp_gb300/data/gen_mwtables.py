"""Generate the multiwavelet filter and cross-correlation tables used by mrcpp_gb300.

The tables are computed from first principles with mpmath (60 digits) and rounded
to IEEE doubles:

* Gauss-Legendre nodes/weights on [0, 1].
* Legendre scaling functions phi_j(x) = sqrt(2j+1) P_j(2x-1) and interpolating
  scaling functions phi_j(x) = sqrt(w_j) sum_m phi^L_m(x_j) phi^L_m(x)
  (the two bases of MRCPP, src/core/LegendreBasis.cpp:60-66 and
  src/core/InterpolatingBasis.cpp:65-86).
* Two-scale filters H0 (scaling) and G0 (wavelet):
  H0_ij = sqrt(2) int_0^1/2 phi_i(x) phi_j(2x) dx,
  G0_ij = sqrt(2) int_0^1/2 psi_i(x) phi_j(2x) dx.
  The wavelets psi_i are Alpert's multiwavelets (B. Alpert, SIAM J. Math. Anal.
  24 (1993) 246): psi_i is orthogonal to all polynomials of degree < K+i on [0,1].
  Each psi_i is unique up to sign; here the sign makes the first non-vanishing
  Legendre moment int psi_i P_{K+i}(2x-1) positive.  H1/G1 follow from the
  symmetry rules of src/core/MWFilter.cpp:225-244 at load time.
  The interpolating wavelets are the Legendre wavelets, so G0^I = G0^L S^T with
  S_jm = sqrt(w_j) phi^L_m(x_j).
* Cross-correlation matrices (operator construction,
  src/treebuilders/CrossCorrelationCalculator.cpp:55-86):
  Left_{i+K*j, p}  = int_0^1 du int_0^u  dv phi_i(u) phi_j(v) phi'_p(1 + v - u)
  Right_{i+K*j, p} = int_0^1 du int_u^1 dv phi_i(u) phi_j(v) phi'_p(v - u)
  where phi' is the scaling basis of order 2k+1.

Output: mwtables.bin next to this script.  Layout (little endian):
  magic 'MWTB' | int32 version=1 | int32 n_entries
  entries: int32 kind (0=H0,1=G0,2=CLEFT,3=CRIGHT) | int32 type (0=Legendre,1=Interpolating)
           int32 order k | int32 rows | int32 cols | rows*cols float64 (row-major)

Run:  python mrcpp_gb300/data/gen_mwtables.py [max_filter_order] [max_cc_order]
"""
import os
import struct
import sys

import mpmath as mp

mp.mp.dps = 60


def gauss_legendre01(n):
    """Gauss-Legendre nodes and weights on [0,1], ascending."""
    xs, ws = [], []
    for i in range(n):
        # Newton iteration on P_n from the Chebyshev-like guess
        z = mp.cos(mp.pi * (i + mp.mpf(3) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p0, p1 = mp.mpf(1), z
            if n == 0:
                break
            for m in range(2, n + 1):
                p0, p1 = p1, ((2 * m - 1) * z * p1 - (m - 1) * p0) / m
            pn = p1 if n >= 1 else mp.mpf(1)
            pnm1 = p0
            dp = n * (z * pn - pnm1) / (z * z - 1)
            dz = pn / dp
            z -= dz
            if abs(dz) < mp.mpf(10) ** (-55):
                break
        # recompute derivative at converged z
        p0, p1 = mp.mpf(1), z
        for m in range(2, n + 1):
            p0, p1 = p1, ((2 * m - 1) * z * p1 - (m - 1) * p0) / m
        dp = n * (z * p1 - p0) / (z * z - 1)
        xs.append((1 - z) / 2)
        ws.append(1 / ((1 - z * z) * dp * dp))
    order = sorted(range(n), key=lambda t: xs[t])
    return [xs[t] for t in order], [ws[t] for t in order]


def legendre_vals(K, x):
    """phi^L_j(x) = sqrt(2j+1) P_j(2x-1), j < K."""
    t = 2 * x - 1
    out = []
    p0, p1 = mp.mpf(1), t
    for j in range(K):
        if j == 0:
            p = p0
        elif j == 1:
            p = p1
        else:
            p = ((2 * j - 1) * t * p1 - (j - 1) * p0) / j
            p0, p1 = p1, p
        out.append(mp.sqrt(2 * j + 1) * p)
    return out


def interp_matrix(K):
    """S_jm = sqrt(w_j) phi^L_m(x_j): interpolating phi^I_j = sum_m S_jm phi^L_m."""
    xs, ws = gauss_legendre01(K)
    return mp.matrix([[mp.sqrt(ws[j]) * legendre_vals(K, xs[j])[m] for m in range(K)] for j in range(K)])


def legendre_filters(K):
    """H0, G0 for the Legendre basis of order k=K-1 (mp matrices)."""
    xs, ws = gauss_legendre01(2 * K + 2)
    # child-0 basis sqrt(2) phi_j(2x) on [0,1/2], child-1 sqrt(2) phi_j(2x-1) on [1/2,1]
    H0 = mp.zeros(K, K)
    H1 = mp.zeros(K, K)
    for a in range(len(xs)):
        x0 = xs[a] / 2
        x1 = (1 + xs[a]) / 2
        w = ws[a] / 2
        par0 = legendre_vals(K, x0)
        par1 = legendre_vals(K, x1)
        ch = legendre_vals(K, xs[a])
        for i in range(K):
            for j in range(K):
                H0[i, j] += mp.sqrt(2) * w * par0[i] * ch[j]
                H1[i, j] += mp.sqrt(2) * w * par1[i] * ch[j]
    # moment matrix: M[m, c] = int P~_m(2x-1) * (child basis function c), m < 2K
    M = mp.zeros(2 * K, 2 * K)
    for a in range(len(xs)):
        x0 = xs[a] / 2
        x1 = (1 + xs[a]) / 2
        w = ws[a] / 2
        p0 = legendre_vals(2 * K, x0)
        p1 = legendre_vals(2 * K, x1)
        ch = legendre_vals(K, xs[a])
        for m in range(2 * K):
            for j in range(K):
                M[m, j] += w * p0[m] * mp.sqrt(2) * ch[j]
                M[m, K + j] += w * p1[m] * mp.sqrt(2) * ch[j]
    # psi_i (coefficient vector over the orthonormal child basis) must satisfy
    # M[m,:] . v = 0 for m < K+i and be orthonormal.  Build from the most
    # constrained (i=K-1) downwards by Gram-Schmidt inside successive null spaces.
    vecs = [None] * K
    for i in range(K - 1, -1, -1):
        ncon = K + i
        A = mp.matrix([[M[m, c] for c in range(2 * K)] for m in range(ncon)])
        # rows of the projector onto the null space of A: use QR of A^T
        Q, _ = mp.qr(A.T, mode='full')
        null = [Q[:, c] for c in range(ncon, 2 * K)]
        # pick the null-space direction orthogonal to all previously built psi
        best = None
        for cand in null:
            v = cand.copy()
            for u in vecs:
                if u is not None:
                    v -= (u.T * v)[0] * u
            if best is None or mp.norm(v) > mp.norm(best):
                best = v
        # Gram-Schmidt the full null space against previous psis and take the
        # component orthogonal to them (the null space has dimension K-i, the
        # previous psi span K-1-i of it)
        basis = []
        for cand in null:
            v = cand.copy()
            for u in vecs:
                if u is not None:
                    v -= (u.T * v)[0] * u
            for u in basis:
                v -= (u.T * v)[0] * u
            nv = mp.norm(v)
            if nv > mp.mpf(10) ** (-30):
                basis.append(v / nv)
        v = basis[0]
        mom = (M[ncon, :] * v)[0] if ncon < 2 * K else mp.mpf(1)
        if mom < 0:
            v = -v
        vecs[i] = v
    G0 = mp.zeros(K, K)
    for i in range(K):
        for j in range(K):
            G0[i, j] = vecs[i][j]
    return H0, G0


def interp_filters(K, H0L, G0L):
    S = interp_matrix(K)
    return S * H0L * S.T, G0L * S.T


def cross_correlation_legendre(k):
    K = k + 1
    Kp = 2 * K  # kernel basis order 2k+1 has 2K functions
    n = 2 * K + 2
    xs, ws = gauss_legendre01(n)
    left = mp.zeros(K * K, Kp)
    right = mp.zeros(K * K, Kp)
    for a in range(n):
        u = xs[a]
        fu = legendre_vals(K, u)
        for b in range(n):
            # left: v in [0,u], kernel argument 1 + v - u in [1-u, 1]
            v = u * xs[b]
            w = ws[a] * ws[b] * u
            fv = legendre_vals(K, v)
            fk = legendre_vals(Kp, 1 + v - u)
            # right: v in [u,1], kernel argument v - u in [0, 1-u]
            v2 = u + (1 - u) * xs[b]
            w2 = ws[a] * ws[b] * (1 - u)
            fv2 = legendre_vals(K, v2)
            fk2 = legendre_vals(Kp, v2 - u)
            for i in range(K):
                for j in range(K):
                    c1 = w * fu[i] * fv[j]
                    c2 = w2 * fu[i] * fv2[j]
                    r = i + K * j
                    for p in range(Kp):
                        left[r, p] += c1 * fk[p]
                        right[r, p] += c2 * fk2[p]
    return left, right


def cross_correlation_interp(k, left, right):
    K = k + 1
    S = interp_matrix(K)
    Sp = interp_matrix(2 * K)
    SS = mp.zeros(K * K, K * K)
    for i in range(K):
        for j in range(K):
            for m in range(K):
                for nn in range(K):
                    SS[i + K * j, m + K * nn] = S[i, m] * S[j, nn]
    return SS * left * Sp.T, SS * right * Sp.T


def to_rows(Mx):
    return [[float(Mx[i, j]) for j in range(Mx.cols)] for i in range(Mx.rows)]


def main():
    max_filter = int(sys.argv[1]) if len(sys.argv) > 1 else 25
    max_cc = int(sys.argv[2]) if len(sys.argv) > 2 else 12
    entries = []
    for k in range(0, max_filter + 1):
        K = k + 1
        H0L, G0L = legendre_filters(K)
        H0I, G0I = interp_filters(K, H0L, G0L)
        entries += [(0, 0, k, to_rows(H0L)), (1, 0, k, to_rows(G0L)),
                    (0, 1, k, to_rows(H0I)), (1, 1, k, to_rows(G0I))]
        print('filters k=%d' % k, flush=True)
    for k in range(1, max_cc + 1):
        L, R = cross_correlation_legendre(k)
        LI, RI = cross_correlation_interp(k, L, R)
        entries += [(2, 0, k, to_rows(L)), (3, 0, k, to_rows(R)),
                    (2, 1, k, to_rows(LI)), (3, 1, k, to_rows(RI))]
        print('cross-correlation k=%d' % k, flush=True)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'mwtables.bin')
    with open(out, 'wb') as fh:
        fh.write(b'MWTB')
        fh.write(struct.pack('<ii', 1, len(entries)))
        for kind, typ, k, rows in entries:
            fh.write(struct.pack('<iiiii', kind, typ, k, len(rows), len(rows[0])))
            for r in rows:
                fh.write(struct.pack('<%dd' % len(r), *r))
    print('wrote', out)


if __name__ == '__main__':
    main()
