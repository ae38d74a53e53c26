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


_lib = None


def build():
    """Compiles liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "oracle_apply.c")):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_apply.restype = C.c_int
        L.oracle_apply.argtypes = [C.POINTER(OracleMra), C.POINTER(OracleOper), C.POINTER(OracleTree), C.POINTER(OracleTree), C.c_double,
                                   C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.oracle_result_info.restype = C.c_int
        L.oracle_result_info.argtypes = [C.c_void_p, _PI, _PD, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong), _PI]
        L.oracle_result_export.restype = C.c_int
        L.oracle_result_export.argtypes = [C.c_void_p, _PI, _PI, _PD, _PD]
        L.oracle_result_free.restype = None
        L.oracle_result_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _pi(a):
    return a.ctypes.data_as(_PI)


def _pd(a):
    return a.ctypes.data_as(_PD)


def apply(prec, out, oper, inp, max_iter=-1, abs_prec=False, nthreads=0, count_terms=True):
    """Oracle apply.  `out` (FunctionTree) gives the starting topology and square
    norm; `oper` a mrcpp_gb300 ConvolutionOperator; `inp` the input FunctionTree.
    Returns a dict with the flat output tree and the counters."""
    mra = inp.mra
    d = mra.desc()
    keep = []
    m = OracleMra()
    m.order, m.root_scale, m.max_scale, m.sf = d.order, d.root_scale, d.max_scale, d.sf
    for i in range(3):
        m.corner[i] = d.corner[i]
        m.nbox[i] = d.nbox[i]
    filt = np.ascontiguousarray(mra._filters)
    keep.append(filt)
    m.filters = _pd(filt)
    ex = oper.export()
    o = OracleOper()
    o.n_terms, o.order, o.build_prec = oper.n_terms, mra.order, float(oper.prec)
    for k in ("depth", "max_transl", "blocks", "norms"):
        keep.append(ex[k])
    o.depth, o.max_transl = _pi(ex["depth"]), _pi(ex["max_transl"])
    o.blocks, o.norms = _pd(ex["blocks"]), _pd(ex["norms"])
    fi = inp.export()
    keep.append(fi)
    ft = OracleTree(len(fi["child0"]), _pi(fi["idx"]), _pi(fi["child0"]), _pd(fi["coefs"]), _pd(fi["norms"]))
    go = out.export()
    keep.append(go)
    gt = OracleTree(len(go["child0"]), _pi(go["idx"]), _pi(go["child0"]), None, None)
    res = C.c_void_p()
    rc = lib().oracle_apply(C.byref(m), C.byref(o), C.byref(ft), C.byref(gt), float(out.square_norm), float(prec), int(max_iter),
                            int(bool(abs_prec)), int(nthreads), int(bool(count_terms)), C.byref(res))
    if rc != 0:
        raise RuntimeError("oracle_apply failed with code %d" % rc)
    n, sq, nt, nc, it = C.c_int(), C.c_double(), C.c_ulonglong(), C.c_ulonglong(), C.c_int()
    lib().oracle_result_info(res, C.byref(n), C.byref(sq), C.byref(nt), C.byref(nc), C.byref(it))
    K3 = mra.kp1 ** 3
    idx = np.zeros((n.value, 4), dtype=np.int32)
    c0 = np.zeros(n.value, dtype=np.int32)
    coefs = np.zeros((n.value, 8 * K3))
    norms = np.zeros((n.value, 8))
    lib().oracle_result_export(res, _pi(idx), _pi(c0), _pd(coefs), _pd(norms))
    lib().oracle_result_free(res)
    return {"idx": idx, "child0": c0, "coefs": coefs, "norms": norms, "square_norm": sq.value, "node_terms": nt.value,
            "components": nc.value, "iterations": it.value}


def to_tree(result, mra):
    """Loads an oracle result into a mrcpp_gb300 FunctionTree (for dot/evalf)."""
    import mrcpp_gb300 as mw
    t = mw.FunctionTree(mra)
    t.load_flat(result["idx"], result["child0"], result["coefs"], result["square_norm"])
    return t
