"""Seeded test cases shared by the tests (inputs of the configurations, at
sizes the CPU oracle finishes in seconds)."""
import numpy as np

import mrcpp_gb300 as mw


def unit_gaussian(beta, center):
    return [((beta / np.pi) ** 1.5, beta, tuple(center))]


def gaussian_sum(seed, n, exp_range, center_range, coef_range=(-1.0, 1.0)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a = float(np.exp(rng.uniform(np.log(exp_range[0]), np.log(exp_range[1]))))
        c = float(rng.uniform(*coef_range))
        r = tuple(float(x) for x in rng.uniform(center_range[0], center_range[1], 3))
        out.append((c, a, r))
    return out


def project(mra, prec, gaussians):
    f = mw.FunctionTree(mra)
    mw.project(prec, f, gaussians)
    return f


def match(gpu_flat, ref):
    """Returns (same_topology, permutation of ref rows onto gpu rows)."""
    key = {tuple(r): i for i, r in enumerate(ref["idx"].tolist())}
    rows = gpu_flat["idx"].tolist()
    if len(rows) != len(key) or any(tuple(r) not in key for r in rows):
        return False, None
    return True, np.array([key[tuple(r)] for r in rows])


def rel_errors(a, b):
    """max |a-b| / max|b| and global relative L2."""
    d = a - b
    return float(np.abs(d).max() / max(np.abs(b).max(), 1e-300)), float(np.linalg.norm(d) / max(np.linalg.norm(b), 1e-300))
