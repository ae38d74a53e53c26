"""CPU oracle for the operator-application path -- TEST INFRASTRUCTURE ONLY.

ctypes binding of oracle/_build/liboracle.so, a plain-C restatement of
mrcpp::apply (see oracle_apply.c for the reference lines it follows).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import this
module; the product package never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
FAST_PATH = os.path.join(HERE, "_build", "liboracle_fast.so")

_PI = C.POINTER(C.c_int)
_PD = C.POINTER(C.c_double)


class OracleMra(C.Structure):
    _fields_ = [("order", C.c_int), ("root_scale", C.c_int), ("corner", C.c_int * 3), ("nbox", C.c_int * 3),
                ("max_scale", C.c_int), ("sf", C.c_double), ("filters", _PD)]


class OracleOper(C.Structure):
    _fields_ = [("n_terms", C.c_int), ("order", C.c_int), ("depth", _PI), ("max_transl", _PI), ("blocks", _PD), ("norms", _PD),
                ("build_prec", C.c_double)]


class OracleTree(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("idx", _PI), ("child0", _PI), ("coefs", _PD), ("norms", _PD)]


_libs = {}


def build():
    """Compiles liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib(fast=False):
    """The checker library, or (fast=True) the same source built with
    -ffast-math, used only to time the CPU baseline."""
    path = FAST_PATH if fast else LIB_PATH
    if path not in _libs:
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(os.path.join(HERE, "oracle_apply.c")):
            build()
        L = C.CDLL(path)
        L.oracle_apply.restype = C.c_int
        L.oracle_apply.argtypes = [C.POINTER(OracleMra), C.POINTER(OracleOper), C.POINTER(OracleTree), C.POINTER(OracleTree), C.c_double,
                                   C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.oracle_apply_sampled.restype = C.c_int
        L.oracle_apply_sampled.argtypes = L.oracle_apply.argtypes[:10] + [C.c_int, C.POINTER(C.c_void_p)]
        L.oracle_apply_prec.restype = C.c_int
        L.oracle_apply_prec.argtypes = L.oracle_apply.argtypes[:10] + [C.c_int, C.c_int, C.POINTER(OracleTree), C.POINTER(C.c_void_p)]
        L.oracle_result_info.restype = C.c_int
        L.oracle_result_info.argtypes = [C.c_void_p, _PI, _PD, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong), _PI]
        L.oracle_result_export.restype = C.c_int
        L.oracle_result_export.argtypes = [C.c_void_p, _PI, _PI, _PD, _PD]
        L.oracle_apply_derivative.restype = C.c_int
        L.oracle_apply_derivative.argtypes = [C.POINTER(OracleMra), C.POINTER(OracleOper), C.POINTER(OracleTree), C.POINTER(OracleTree), C.c_int,
                                              C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.oracle_combine.restype = C.c_int
        L.oracle_combine.argtypes = [C.POINTER(OracleMra), C.c_int, C.c_int, C.POINTER(OracleTree), _PD, _PD, _PD, C.POINTER(OracleTree),
                                     C.c_double, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.oracle_combine_ex.restype = C.c_int
        L.oracle_combine_ex.argtypes = L.oracle_combine.argtypes[:11] + [C.c_int, C.POINTER(C.c_void_p)]
        L.oracle_project.restype = C.c_int
        L.oracle_project.argtypes = [C.POINTER(OracleMra), _PD, _PD, C.POINTER(OracleTree), C.c_double, C.c_int, C.c_int, _ORACLE_FUNC, C.c_void_p,
                                     C.POINTER(C.c_void_p)]
        L.oracle_result_free.restype = None
        L.oracle_result_free.argtypes = [C.c_void_p]
        _libs[path] = L
    return _libs[path]


def _pi(a):
    return a.ctypes.data_as(_PI)


def _pd(a):
    return a.ctypes.data_as(_PD)


class Prepared:
    """Marshalled inputs of one oracle apply; run() calls the C oracle only
    (so a timing of run() covers the restated reference path alone).

    Prepared(prec, out, oper, inp) takes mrcpp_gb300 objects; from_arrays()
    takes plain arrays (so that a process can run the oracle without loading
    the library under test)."""

    def __init__(self, prec, out, oper, inp, max_iter=-1, abs_prec=False, prec_trees=None):
        d = inp.mra.desc()
        mra = {"order": d.order, "root_scale": d.root_scale, "max_scale": d.max_scale, "sf": d.sf, "corner": [d.corner[i] for i in range(3)],
               "nbox": [d.nbox[i] for i in range(3)], "filters": inp.mra._filters}
        ex = oper.export()
        op = {"n_terms": oper.n_terms, "build_prec": float(getattr(oper, "prec", 1.0)), "depth": ex["depth"], "max_transl": ex["max_transl"],
              "blocks": ex["blocks"], "norms": ex["norms"]}
        pts = None if prec_trees is None else [t.export() for t in prec_trees]
        self._setup(prec, mra, op, inp.export(), out.export(), float(out.square_norm), max_iter, abs_prec, pts)

    @classmethod
    def from_arrays(cls, prec, mra, oper, inp, out, out_sqnorm=-1.0, max_iter=-1, abs_prec=False, prec_trees=None):
        """mra: order, root_scale, max_scale, sf, corner[3], nbox[3], filters;
        oper: n_terms, build_prec, depth, max_transl, blocks, norms; inp: idx,
        child0, coefs, norms; out: idx, child0 (the starting topology);
        prec_trees: trees like inp (the precTrees form of apply)."""
        self = cls.__new__(cls)
        self._setup(prec, mra, oper, inp, out, out_sqnorm, max_iter, abs_prec, prec_trees)
        return self

    @staticmethod
    def _tree(t, keep):
        a = {"idx": np.ascontiguousarray(t["idx"], dtype=np.int32), "child0": np.ascontiguousarray(t["child0"], dtype=np.int32),
             "coefs": np.ascontiguousarray(t["coefs"], dtype=np.float64), "norms": np.ascontiguousarray(t["norms"], dtype=np.float64)}
        keep.append(a)
        return OracleTree(len(a["child0"]), _pi(a["idx"]), _pi(a["child0"]), _pd(a["coefs"]), _pd(a["norms"]))

    def _setup(self, prec, mra, oper, inp, out, out_sqnorm, max_iter, abs_prec, prec_trees=None):
        self.prec, self.max_iter, self.abs_prec = float(prec), int(max_iter), int(bool(abs_prec))
        self.kp1 = int(mra["order"]) + 1
        self.keep = []
        m = OracleMra()
        m.order, m.root_scale, m.max_scale, m.sf = int(mra["order"]), int(mra["root_scale"]), int(mra["max_scale"]), float(mra["sf"])
        for i in range(3):
            m.corner[i] = int(mra["corner"][i])
            m.nbox[i] = int(mra["nbox"][i])
        filt = np.ascontiguousarray(mra["filters"], dtype=np.float64)
        self.keep.append(filt)
        m.filters = _pd(filt)
        o = OracleOper()
        o.n_terms, o.order, o.build_prec = int(oper["n_terms"]), int(mra["order"]), float(oper["build_prec"])
        arrs = {k: np.ascontiguousarray(oper[k], dtype=np.int32 if k in ("depth", "max_transl") else np.float64)
                for k in ("depth", "max_transl", "blocks", "norms")}
        self.keep.append(arrs)
        o.depth, o.max_transl = _pi(arrs["depth"]), _pi(arrs["max_transl"])
        o.blocks, o.norms = _pd(arrs["blocks"]), _pd(arrs["norms"])
        ft = self._tree(inp, self.keep)
        self.n_prec = 0 if prec_trees is None else len(prec_trees)
        self.pt = (OracleTree * max(self.n_prec, 1))(*[self._tree(t, self.keep) for t in (prec_trees or [])])
        go = {"idx": np.ascontiguousarray(out["idx"], dtype=np.int32), "child0": np.ascontiguousarray(out["child0"], dtype=np.int32)}
        self.keep.append(go)
        gt = OracleTree(len(go["child0"]), _pi(go["idx"]), _pi(go["child0"]), None, None)
        self.m, self.o, self.ft, self.gt = m, o, ft, gt
        self.out_sqnorm = float(out_sqnorm)

    def run(self, nthreads=0, count_terms=True, sample=1, export=True, fast=False, deriv_dir=None, deriv_order=1):
        L = lib(fast)
        res = C.c_void_p()
        if deriv_dir is None:
            rc = L.oracle_apply_prec(C.byref(self.m), C.byref(self.o), C.byref(self.ft), C.byref(self.gt), self.out_sqnorm, self.prec,
                                     self.max_iter, self.abs_prec, int(nthreads), int(bool(count_terms)), int(sample), self.n_prec, self.pt,
                                     C.byref(res))
        else:
            rc = L.oracle_apply_derivative(C.byref(self.m), C.byref(self.o), C.byref(self.ft), C.byref(self.gt), int(deriv_dir),
                                           int(deriv_order), int(nthreads), C.byref(res))
        if rc != 0:
            raise RuntimeError("oracle_apply failed with code %d" % rc)
        n, sq, nt, nc, it = C.c_int(), C.c_double(), C.c_ulonglong(), C.c_ulonglong(), C.c_int()
        L.oracle_result_info(res, C.byref(n), C.byref(sq), C.byref(nt), C.byref(nc), C.byref(it))
        out = {"square_norm": sq.value, "node_terms": nt.value, "components": nc.value, "iterations": it.value, "n_nodes": n.value}
        if export:
            K3 = self.kp1 ** 3
            out["idx"] = np.zeros((n.value, 4), dtype=np.int32)
            out["child0"] = np.zeros(n.value, dtype=np.int32)
            out["coefs"] = np.zeros((n.value, 8 * K3))
            out["norms"] = np.zeros((n.value, 8))
            L.oracle_result_export(res, _pi(out["idx"]), _pi(out["child0"]), _pd(out["coefs"]), _pd(out["norms"]))
        L.oracle_result_free(res)
        return out


def apply(prec, out, oper, inp, max_iter=-1, abs_prec=False, nthreads=0, count_terms=True, sample=1, prec_trees=None):
    """Oracle apply.  `out` (FunctionTree) gives the starting topology and square
    norm; `oper` a mrcpp_gb300 ConvolutionOperator; `inp` the input FunctionTree;
    `prec_trees` (FunctionTrees) selects the precTrees form of apply.
    Returns a dict with the flat output tree and the counters."""
    return Prepared(prec, out, oper, inp, max_iter, abs_prec, prec_trees).run(nthreads, count_terms, sample)


def apply_derivative(out, oper, inp, dir, nthreads=0):
    """Oracle apply(out, DerivativeOperator, inp, dir), of the operator's order
    (`oper.order`, 1 when absent): `out` holds only its roots; returns the flat
    copy-adapted output tree."""
    return Prepared(1.0, out, oper, inp).run(nthreads, deriv_dir=dir, deriv_order=getattr(oper, "order", 1))


_ORACLE_FUNC = C.CFUNCTYPE(None, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)


def basis_maps(basis, order):
    """Quadrature roots on [0, 1] and the value-to-coefficient map of the
    scaling basis, computed here with numpy (LegendreBasis::calcCVMaps,
    LegendreBasis.cpp:98-109: vcMap(i, k) = phi_k(x_i) w_i with phi_k =
    sqrt(2k+1) P_k(2x - 1); InterpolatingBasis::calcCVMaps,
    InterpolatingBasis.cpp:115-123: vcMap(k, k) = sqrt(w_k)); column-major."""
    from numpy.polynomial import legendre as npleg

    K = order + 1
    x, w = npleg.leggauss(K)
    x, w = 0.5 * (x + 1.0), 0.5 * w
    vc = np.zeros((K, K))
    if basis == 0:  # Legendre
        for k in range(K):
            c = np.zeros(k + 1)
            c[k] = 1.0
            vc[:, k] = np.sqrt(2 * k + 1) * npleg.legval(2 * x - 1, c) * w
    else:
        vc[np.arange(K), np.arange(K)] = np.sqrt(w)
    return x, np.ascontiguousarray(vc.T).ravel()  # element (i, k) at i + K k


def project(prec, tree, func, max_iter=-1, abs_prec=False):
    """Oracle project(prec, tree, func) from the current grid of `tree` (a
    FunctionTree; only its MRA and node indices are read): func takes an (n, 3)
    array of points and returns n values.  Returns the flat result tree."""
    mra = tree.mra
    d = mra.desc()
    m = OracleMra()
    m.order, m.root_scale, m.max_scale, m.sf = d.order, d.root_scale, d.max_scale, d.sf
    for i in range(3):
        m.corner[i] = d.corner[i]
        m.nbox[i] = d.nbox[i]
    filt = np.ascontiguousarray(mra._filters)
    m.filters = _pd(filt)
    roots, vc = basis_maps(mra.basis, mra.order)
    go = tree.export()
    gt = OracleTree(len(go["child0"]), _pi(go["idx"]), _pi(go["child0"]), None, None)
    errors = []

    def cb(n, r, v, _user):
        try:
            pts = np.ctypeslib.as_array(r, shape=(n, 3))
            np.ctypeslib.as_array(v, shape=(n,))[:] = np.asarray(func(pts), dtype=np.float64).reshape(n)
        except BaseException as e:
            errors.append(e)

    f = _ORACLE_FUNC(cb)
    res = C.c_void_p()
    L = lib()
    rc = L.oracle_project(C.byref(m), _pd(vc), _pd(roots), C.byref(gt), float(prec), int(max_iter), int(bool(abs_prec)), f, None, C.byref(res))
    if errors:
        raise errors[0]
    if rc != 0:
        raise RuntimeError("oracle_project failed with code %d" % rc)
    return _export_result(L, res, mra.kp1)


def combine(op, prec, out, terms, max_iter=-1, abs_prec=False, use_max_norms=False):
    """Oracle add (op 0) / multiply (op 1) of terms [(c, FunctionTree), ...] from
    the grid of `out` (use_max_norms: multiply's max-norm adaptor); returns the
    flat result tree."""
    mra = out.mra
    d = mra.desc()
    m = OracleMra()
    m.order, m.root_scale, m.max_scale, m.sf = d.order, d.root_scale, d.max_scale, d.sf
    for i in range(3):
        m.corner[i] = d.corner[i]
        m.nbox[i] = d.nbox[i]
    filt = np.ascontiguousarray(mra._filters)
    m.filters = _pd(filt)
    keep = [filt]
    trees = (OracleTree * len(terms))()
    for j, (_, t) in enumerate(terms):
        x = t.export()
        keep.append(x)
        trees[j] = OracleTree(len(x["child0"]), _pi(x["idx"]), _pi(x["child0"]), _pd(x["coefs"]), _pd(x["norms"]))
    c = np.ascontiguousarray([float(t[0]) for t in terms])
    cv, vc, _, _ = mra.maps()
    go = out.export()
    gt = OracleTree(len(go["child0"]), _pi(go["idx"]), _pi(go["child0"]), None, None)
    res = C.c_void_p()
    L = lib()
    rc = L.oracle_combine_ex(C.byref(m), int(op), len(terms), trees, _pd(c), _pd(cv), _pd(vc), C.byref(gt), float(prec), int(max_iter),
                             int(bool(abs_prec)), int(bool(use_max_norms)), C.byref(res))
    if rc != 0:
        raise RuntimeError("oracle_combine failed with code %d" % rc)
    return _export_result(L, res, mra.kp1)


def _export_result(L, res, kp1):
    n, sq, nt, nc, it = C.c_int(), C.c_double(), C.c_ulonglong(), C.c_ulonglong(), C.c_int()
    L.oracle_result_info(res, C.byref(n), C.byref(sq), C.byref(nt), C.byref(nc), C.byref(it))
    K3 = kp1 ** 3
    out_ = {"square_norm": sq.value, "iterations": it.value, "n_nodes": n.value, "idx": np.zeros((n.value, 4), dtype=np.int32),
            "child0": np.zeros(n.value, dtype=np.int32), "coefs": np.zeros((n.value, 8 * K3)), "norms": np.zeros((n.value, 8))}
    L.oracle_result_export(res, _pi(out_["idx"]), _pi(out_["child0"]), _pd(out_["coefs"]), _pd(out_["norms"]))
    L.oracle_result_free(res)
    return out_


def to_tree(result, mra):
    """Loads an oracle result into a mrcpp_gb300 FunctionTree (for dot/evalf)."""
    import mrcpp_gb300 as mw
    t = mw.FunctionTree(mra)
    t.load_flat(result["idx"], result["child0"], result["coefs"], result["square_norm"])
    return t
