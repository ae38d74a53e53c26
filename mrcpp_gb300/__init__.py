"""mrcpp_gb300: GB300-native multiwavelet operator application.

Python mirror of the MRCPP interface for the operator-application path
(``mrcpp::apply`` with ``PoissonOperator`` / ``HelmholtzOperator``), bound
with ctypes to ``libmwgpu.so``.  The library holds the sm_103a CUDA kernels
behind the C-ABI of ``include/mwgpu.h`` and the C++ host mirror of
``include/mwhost.h`` (MRA, FunctionTree, projection, operator construction).

There is no CPU implementation of the operator application here: ``apply``
always runs on the GPU and raises ``MWGPUError`` when no device or no library
is available.
"""
import ctypes as C
import os

import numpy as np

__all__ = [
    "MWGPUError", "lib", "MRA", "FunctionTree", "PoissonOperator", "HelmholtzOperator", "ConvolutionOperator",
    "build_grid", "project", "apply", "apply_batch", "apply_learned", "GridNetwork", "grid_features", "copy_grid", "dot", "poisson_kernel", "helmholtz_kernel",
    "LEGENDRE", "INTERPOLATING", "FP64", "MIXED",
]

LEGENDRE = 0
INTERPOLATING = 1
FP64 = 0
MIXED = 1

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmwgpu.so")


class MWGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("mwgpu error %d: %s" % (code, msg))
        self.code = code


class MwgpuMraDesc(C.Structure):
    _fields_ = [("order", C.c_int), ("root_scale", C.c_int), ("corner", C.c_int * 3), ("nbox", C.c_int * 3),
                ("max_scale", C.c_int), ("sf", C.c_double), ("filters", C.POINTER(C.c_double))]


class MwgpuOperDesc(C.Structure):
    _fields_ = [("n_terms", C.c_int), ("order", C.c_int), ("depth", C.POINTER(C.c_int)), ("max_transl", C.POINTER(C.c_int)),
                ("blocks", C.POINTER(C.c_double)), ("norms", C.POINTER(C.c_double)), ("build_prec", C.c_double)]


class MwgpuTreeDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("idx", C.POINTER(C.c_int)), ("child0", C.POINTER(C.c_int)),
                ("coefs", C.POINTER(C.c_double)), ("norms", C.POINTER(C.c_double))]


class MwgpuConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("reserved", C.c_int * 6)]


class MwgpuLevelStats(C.Structure):
    _fields_ = [("node_terms", C.c_ulonglong), ("components", C.c_ulonglong), ("band_nodes", C.c_ulonglong),
                ("gen_nodes", C.c_ulonglong), ("device_ms", C.c_double), ("contract_ms", C.c_double)]


class MwhApplyStats(C.Structure):
    _fields_ = [("node_terms", C.c_ulonglong), ("components", C.c_ulonglong), ("band_nodes", C.c_ulonglong),
                ("gen_nodes", C.c_ulonglong), ("iterations", C.c_int), ("out_nodes", C.c_int), ("device_ms", C.c_double),
                ("contract_ms", C.c_double), ("transform_ms", C.c_double), ("wall_ms", C.c_double),
                ("launches", C.c_ulonglong), ("h2d_bytes", C.c_ulonglong), ("d2h_bytes", C.c_ulonglong), ("planned", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MwhLearnedStats(C.Structure):
    _fields_ = [("apply", MwhApplyStats), ("proposal_nodes", C.c_int), ("proposal_levels", C.c_int), ("kept_nodes", C.c_int),
                ("first_miss", C.c_int), ("fallback", C.c_int), ("host_round_trips", C.c_int), ("predict_ms", C.c_double),
                ("judged_ms", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "apply"}
        d["apply"] = self.apply.as_dict()
        return d


_P = C.c_void_p
_PI = C.POINTER(C.c_int)
_PD = C.POINTER(C.c_double)
_PF = C.POINTER(C.c_float)
_SIGS = {
    # device C-ABI (include/mwgpu.h)
    "mwgpu_init": (C.c_int, [C.POINTER(_P), C.POINTER(MwgpuConfig)]),
    "mwgpu_destroy": (C.c_int, [_P]),
    "mwgpu_last_error": (C.c_char_p, [_P]),
    "mwgpu_set_precision": (C.c_int, [_P, C.c_int]),
    "mwgpu_upload_operator": (C.c_int, [_P, C.POINTER(MwgpuMraDesc), C.POINTER(MwgpuOperDesc), C.c_double, C.POINTER(_P)]),
    "mwgpu_free_operator": (C.c_int, [_P, _P]),
    "mwgpu_operator_bandwidths": (C.c_int, [_P, _P, _PI, _PI, _PI]),
    "mwgpu_upload_tree": (C.c_int, [_P, C.POINTER(MwgpuMraDesc), C.POINTER(MwgpuTreeDesc), C.POINTER(_P)]),
    "mwgpu_create_tree": (C.c_int, [_P, C.POINTER(MwgpuMraDesc), C.POINTER(MwgpuTreeDesc), C.POINTER(_P)]),
    "mwgpu_tree_add_nodes": (C.c_int, [_P, _P, C.c_int, _PI, C.c_int, _PI, _PI]),
    "mwgpu_tree_size": (C.c_int, [_P, _PI]),
    "mwgpu_free_tree": (C.c_int, [_P, _P]),
    "mwgpu_apply_level": (C.c_int, [_P, _P, _P, _P, _PI, C.c_int, C.c_double, C.c_double, _PD, C.POINTER(MwgpuLevelStats)]),
    "mwgpu_apply_level_scaled": (C.c_int, [_P, _P, _P, _P, _PI, C.c_int, C.c_double, C.c_double, _PD, _PD, C.POINTER(MwgpuLevelStats)]),
    "mwgpu_apply_derivative": (C.c_int, [_P, _P, _P, _P, _PI, C.c_int, C.c_int, C.c_int, C.POINTER(MwgpuLevelStats)]),
    "mwgpu_transform": (C.c_int, [_P, _P, C.c_int, C.c_int]),
    "mwgpu_apply_level_batch": (C.c_int, [_P, _P, C.c_int, C.POINTER(_P), C.POINTER(_P), _PI, _PI, C.c_int, C.c_double, _PD, _PD,
                                          C.POINTER(MwgpuLevelStats)]),
    "mwgpu_transform_batch": (C.c_int, [_P, C.c_int, C.POINTER(_P), C.c_int, C.c_int]),
    "mwgpu_plan_create": (C.c_int, [_P, _P, C.c_int, C.POINTER(_P), C.POINTER(_P), _PI, _PI, C.c_int, C.c_double, _PD, C.c_int,
                                    C.POINTER(_P)]),
    "mwgpu_plan_execute": (C.c_int, [_P, _P, C.POINTER(MwgpuLevelStats)]),
    "mwgpu_plan_check": (C.c_int, [_P, _P, C.POINTER(MwgpuLevelStats)]),
    "mwgpu_plan_info": (C.c_int, [_P, C.POINTER(C.c_longlong), _PI, _PI, C.POINTER(C.c_longlong), _PD, C.POINTER(C.c_ulonglong)]),
    "mwgpu_plan_pencil_info": (C.c_int, [_P, C.POINTER(C.c_ulonglong), _PD]),
    "mwgpu_plan_tuning": (C.c_int, [_P, _PI, C.POINTER(C.c_longlong), _PI, _PD, _PI]),
    "mwgpu_fp64_pipe_rates": (C.c_int, [_P, _PD, _PD]),
    "mwgpu_plan_destroy": (C.c_int, [_P, _P]),
    "mwgpu_tree_update_coefs": (C.c_int, [_P, _P, _PD, _PD]),
    "mwgpu_apply_judged": (C.c_int, [_P, _P, _P, _P, C.c_int, _PI, C.c_double, C.c_int, C.c_int, _PD, C.c_int, _PI, _PI, _PD,
                                     C.POINTER(MwgpuLevelStats)]),
    "mwgpu_mlp_create": (C.c_int, [_P, _PF, C.POINTER(_P)]),
    "mwgpu_mlp_destroy": (C.c_int, [_P, _P]),
    "mwgpu_mlp_get": (C.c_int, [_P, _P, _PF, C.POINTER(C.c_uint16)]),
    "mwgpu_mlp_features": (C.c_int, [_P, _P, _P, C.c_double, _PI, C.c_int, _PF]),
    "mwgpu_mlp_infer": (C.c_int, [_P, _P, _PF, C.c_int, _PF]),
    "mwgpu_mlp_predict": (C.c_int, [_P, _P, _P, _P, C.c_double, _PI, C.c_int, _PF]),
    "mwgpu_tree_copy_nodes": (C.c_int, [_P, _P, _P, C.c_int, _PI, _PI]),
    "mwgpu_mlp_grad": (C.c_int, [_P, _P, _PF, _PF, C.c_int, C.c_float, _PF, _PF]),
    "mwgpu_mlp_train": (C.c_int, [_P, _P, _PF, _PF, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_uint, _PF]),
    "mwgpu_download_tree": (C.c_int, [_P, _P, _PD, _PD]),
    "mwgpu_download_nodes": (C.c_int, [_P, _P, C.c_int, _PI, _PD, _PD]),
    "mwgpu_sync": (C.c_int, [_P]),
    "mwgpu_tree_clear_generated": (C.c_int, [_P, _P]),
    "mwgpu_timer_mark": (C.c_int, [_P, C.c_int]),
    "mwgpu_timer_elapsed": (C.c_int, [_P, C.c_int, C.c_int, _PD]),
    "mwgpu_launch_count": (C.c_int, [_P, C.POINTER(C.c_ulonglong)]),
    "mwgpu_scrub_l2": (C.c_int, [_P, C.c_size_t]),
    # host mirror (include/mwhost.h)
    "mwh_last_error": (C.c_char_p, []),
    "mwh_set_table_path": (C.c_int, [C.c_char_p]),
    "mwh_mra_create": (C.c_int, [C.c_int, C.c_int, C.c_int, _PI, _PI, C.c_double, C.c_int, C.POINTER(_P)]),
    "mwh_mra_from_bounds": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_P)]),
    "mwh_mra_free": (None, [_P]),
    "mwh_mra_desc": (C.c_int, [_P, C.POINTER(MwgpuMraDesc), _PD]),
    "mwh_mra_maps": (C.c_int, [_P, _PD, _PD, _PD, _PD]),
    "mwh_tree_create": (C.c_int, [_P, C.POINTER(_P)]),
    "mwh_tree_free": (None, [_P]),
    "mwh_pinned_stats": (C.c_int, [C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]),
    "mwh_build_grid_gauss": (C.c_int, [_P, C.c_int, _PD, _PD, _PD]),
    "mwh_project_gauss": (C.c_int, [C.c_double, _P, C.c_int, _PD, _PD, _PD, C.c_int, C.c_int]),
    "mwh_project_func": (C.c_int, [C.c_double, _P, C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "mwh_project_func_device": (C.c_int, [C.c_double, _P, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(MwhApplyStats)]),
    "mwgpu_project_level_values": (C.c_int, [_P, _P, _PD, _PD, _PD, _PI, C.c_int, _PD]),
    "mwh_tree_rescale": (C.c_int, [_P, C.c_double]),
    "mwh_convolution": (C.c_int, [_P, C.c_int, _PD, _PD, C.c_double, C.POINTER(_P)]),
    "mwh_mra_distances": (C.c_int, [_P, C.c_double, _PD, _PD]),
    "mwh_copy_grid": (C.c_int, [_P, _P]),
    "mwh_add": (C.c_int, [C.c_double, _P, C.c_int, _PD, C.POINTER(_P), C.c_int, C.c_int, C.POINTER(MwhApplyStats)]),
    "mwh_multiply": (C.c_int, [C.c_double, _P, C.c_int, _PD, C.POINTER(_P), C.c_int, C.c_int, C.POINTER(MwhApplyStats)]),
    "mwh_multiply_max_norms": (C.c_int, [C.c_double, _P, C.c_int, _PD, C.POINTER(_P), C.c_int, C.POINTER(MwhApplyStats)]),
    "mwgpu_combine_level": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(_P), _PD, _PD, _PD, _P, _PI, C.c_int, _PD]),
    "mwh_project_gauss_device": (C.c_int, [C.c_double, _P, C.c_int, _PD, _PD, _PD, C.c_int, C.c_int, C.POINTER(MwhApplyStats)]),
    "mwgpu_project_level": (C.c_int, [_P, _P, C.c_int, _PD, _PD, _PD, _PI, C.c_int, _PD]),
    "mwh_tree_info": (C.c_int, [_P, _PI, _PD]),
    "mwh_tree_export": (C.c_int, [_P, _PI, _PI, _PD, _PD]),
    "mwh_tree_import": (C.c_int, [_P, C.c_int, _PI, _PI, _PD, C.c_double]),
    "mwh_tree_save": (C.c_int, [_P, C.c_char_p]),
    "mwh_tree_load": (C.c_int, [_P, C.c_char_p]),
    "mwh_dot": (C.c_double, [_P, _P]),
    "mwh_evalf": (C.c_double, [_P, C.c_double, C.c_double, C.c_double]),
    "mwh_integrate": (C.c_double, [_P]),
    "mwh_poisson": (C.c_int, [_P, C.c_double, C.POINTER(_P)]),
    "mwh_helmholtz": (C.c_int, [_P, C.c_double, C.c_double, C.POINTER(_P)]),
    "mwh_abgv": (C.c_int, [_P, C.c_double, C.c_double, C.POINTER(_P)]),
    "mwh_apply_derivative": (C.c_int, [_P, _P, _P, C.c_int, C.POINTER(MwhApplyStats)]),
    "mwh_oper_free": (None, [_P]),
    "mwh_oper_info": (C.c_int, [_P, _PI, _PI, _PI]),
    "mwh_oper_export": (C.c_int, [_P, _PI, _PI, _PD, _PD, _PD, _PD]),
    "mwh_oper_desc": (C.c_int, [_P, C.POINTER(MwgpuOperDesc)]),
    "mwh_poisson_kernel": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_int, _PD, _PD]),
    "mwh_helmholtz_kernel": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _PD, _PD]),
    "mwh_apply": (C.c_int, [C.c_double, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.POINTER(MwhApplyStats)]),
    "mwh_ph": (C.c_int, [_P, C.c_int, C.c_char_p, C.POINTER(_P)]),
    "mwh_bs": (C.c_int, [_P, C.c_int, C.c_char_p, C.POINTER(_P)]),
    "mwh_deriv_tables": (C.c_int, [_P, C.c_int, _PD, _PD, _PD, C.POINTER(_P)]),
    "mwh_apply_prec": (C.c_int, [C.c_double, _P, _P, _P, C.c_int, _P, C.c_int, C.c_int, C.c_int, C.POINTER(MwhApplyStats)]),
    "mwh_prec_factors": (C.c_int, [C.c_int, _P, C.c_int, _PI, _PD]),
    "mwh_apply_batch": (C.c_int, [C.c_double, C.c_int, C.POINTER(_P), _P, C.POINTER(_P), C.c_int, C.c_int, C.c_int,
                                  C.POINTER(MwhApplyStats)]),
    "mwh_mlp_create": (C.c_int, [_PF, C.POINTER(_P)]),
    "mwh_mlp_free": (None, [_P]),
    "mwh_apply_learned": (C.c_int, [C.c_double, _P, _P, _P, _P, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(MwhLearnedStats)]),
    "mwh_grid_features": (C.c_int, [C.c_double, _P, _P, _P, _PF, _PF]),
}

_lib = None


def lib():
    """The loaded libmwgpu.so (raises MWGPUError if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MWGPUError(6, "libmwgpu.so not built (%s); run python -m mrcpp_gb300.build" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ck(code):
    if code != 0:
        raise MWGPUError(code, lib().mwh_last_error().decode())


def _pi(a):
    return a.ctypes.data_as(_PI)


def _pd(a):
    return a.ctypes.data_as(_PD)


class MRA:
    """MultiResolutionAnalysis<3>: world box + scaling basis (src/trees/MultiResolutionAnalysis.h)."""

    def __init__(self, box=(-20, 20), order=5, basis=INTERPOLATING, max_depth=30, scale=None, corner=None, nbox=None, sf=None):
        h = _P()
        if scale is not None:
            c = np.ascontiguousarray(corner, dtype=np.int32)
            nb = np.ascontiguousarray(nbox, dtype=np.int32)
            _ck(lib().mwh_mra_create(basis, order, scale, _pi(c), _pi(nb), float(sf if sf else 1.0), max_depth, C.byref(h)))
        else:
            _ck(lib().mwh_mra_from_bounds(basis, order, int(box[0]), int(box[1]), max_depth, C.byref(h)))
        self._h = h
        self.order = order
        self.kp1 = order + 1
        self.basis = basis
        self._desc = MwgpuMraDesc()
        self._filters = np.zeros(8 * self.kp1 * self.kp1)
        _ck(lib().mwh_mra_desc(self._h, C.byref(self._desc), _pd(self._filters)))
        self.root_scale = self._desc.root_scale
        self.corner = tuple(self._desc.corner)
        self.nbox = tuple(self._desc.nbox)
        self.sf = self._desc.sf
        self.max_scale = self._desc.max_scale

    def calcMinDistance(self, eps):
        """sqrt(eps 2^-maxScale) (MultiResolutionAnalysis.h:65)."""
        r = C.c_double()
        _ck(lib().mwh_mra_distances(self._h, float(eps), C.byref(r), None))
        return r.value

    def calcMaxDistance(self):
        """Diagonal of the world box (MultiResolutionAnalysis::calcMaxDistance)."""
        r = C.c_double()
        _ck(lib().mwh_mra_distances(self._h, 1.0, None, C.byref(r)))
        return r.value

    def maps(self):
        """(cv_map, vc_map, roots, weights) of the scaling basis; the maps K x K column-major."""
        K = self.kp1
        cv, vc, r, w = np.zeros(K * K), np.zeros(K * K), np.zeros(K), np.zeros(K)
        _ck(lib().mwh_mra_maps(self._h, _pd(cv), _pd(vc), _pd(r), _pd(w)))
        return cv, vc, r, w

    @property
    def filters(self):
        """8 (k+1)x(k+1) column-major filters: compression H0t,H1t,G0t,G1t, reconstruction H0,G0,H1,G1."""
        K = self.kp1
        return self._filters.reshape(8, K, K).transpose(0, 2, 1).copy()  # [f][row][col]

    def desc(self):
        return self._desc

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mwh_mra_free(self._h)
            self._h = None


class FunctionTree:
    """FunctionTree<3>: adaptive tree of compressed s+d node coefficients."""

    def __init__(self, mra):
        self.mra = mra
        h = _P()
        _ck(lib().mwh_tree_create(mra._h, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mwh_tree_free(self._h)
            self._h = None

    @property
    def n_nodes(self):
        n = C.c_int()
        _ck(lib().mwh_tree_info(self._h, C.byref(n), None))
        return n.value

    @property
    def square_norm(self):
        s = C.c_double()
        _ck(lib().mwh_tree_info(self._h, None, C.byref(s)))
        return s.value

    def export(self):
        """Flat breadth-first copy: idx [n,4], child0 [n], coefs [n, 8K^3], norms [n, 8]."""
        n = self.n_nodes
        K3 = self.mra.kp1 ** 3
        idx = np.zeros((n, 4), dtype=np.int32)
        c0 = np.zeros(n, dtype=np.int32)
        coefs = np.zeros((n, 8 * K3))
        norms = np.zeros((n, 8))
        _ck(lib().mwh_tree_export(self._h, _pi(idx), _pi(c0), _pd(coefs), _pd(norms)))
        return {"idx": idx, "child0": c0, "coefs": coefs, "norms": norms}

    def load_flat(self, idx, child0, coefs, square_norm=-1.0):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        c0 = np.ascontiguousarray(child0, dtype=np.int32)
        coefs = np.ascontiguousarray(coefs, dtype=np.float64)
        _ck(lib().mwh_tree_import(self._h, len(c0), _pi(idx), _pi(c0), _pd(coefs), float(square_norm)))

    def saveTree(self, file):
        """FunctionTree::saveTree: writes `file` + ".mwtree" (flat, versioned layout)."""
        _ck(lib().mwh_tree_save(self._h, os.fsencode(file)))

    def loadTree(self, file):
        """FunctionTree::loadTree: reads `file` + ".mwtree"; the tree's MRA must be the file's."""
        _ck(lib().mwh_tree_load(self._h, os.fsencode(file)))

    def evalf(self, r):
        return lib().mwh_evalf(self._h, float(r[0]), float(r[1]), float(r[2]))

    def integrate(self):
        return lib().mwh_integrate(self._h)

    def rescale(self, c):
        """FunctionTree::rescale(c) (src/trees/FunctionTree.cpp:651-668)."""
        _ck(lib().mwh_tree_rescale(self._h, float(c)))


def _gauss_arrays(gaussians):
    coef = np.ascontiguousarray([g[0] for g in gaussians], dtype=np.float64)
    ex = np.ascontiguousarray([g[1] for g in gaussians], dtype=np.float64)
    pos = np.ascontiguousarray([list(g[2]) for g in gaussians], dtype=np.float64).reshape(-1)
    return coef, ex, pos


def build_grid(tree, gaussians):
    """build_grid(tree, GaussExp): gaussians = [(coef, exponent, (x,y,z)), ...]."""
    coef, ex, pos = _gauss_arrays(gaussians)
    _ck(lib().mwh_build_grid_gauss(tree._h, len(coef), _pd(coef), _pd(ex), _pd(pos)))


_FUNC = C.CFUNCTYPE(None, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)


def _project_func(prec, tree, func, max_iter, abs_prec, device=False):
    errors = []

    def cb(n, r, v, _user):
        try:
            pts = np.ctypeslib.as_array(r, shape=(n, 3))
            out = np.ctypeslib.as_array(v, shape=(n,))
            out[:] = np.asarray(func(pts), dtype=np.float64).reshape(n)
        except BaseException as e:  # reported after the C call returns
            errors.append(e)

    f = _FUNC(cb)
    st = MwhApplyStats()
    if device:
        code = lib().mwh_project_func_device(float(prec), tree._h, C.cast(f, C.c_void_p), None, int(max_iter), int(bool(abs_prec)), C.byref(st))
    else:
        code = lib().mwh_project_func(float(prec), tree._h, C.cast(f, C.c_void_p), None, int(max_iter), int(bool(abs_prec)))
    if errors:
        raise errors[0]
    _ck(code)
    return st.as_dict() if device else None


def project(prec, tree, gaussians, max_iter=-1, abs_prec=False, grid=True, device=False):
    """build_grid (optional) + project(prec, tree, GaussExp) (src/treebuilders/project.cpp:41-66).
    device=True computes the nodes on the GPU (mwgpu_project_level) and returns
    the statistics; the default projects on the host like the reference.

    gaussians may also be a function: project(prec, tree, func) with func
    taking an (n, 3) array of points and returning n values is
    project(prec, tree, std::function) (project.cpp:59-63), from the tree's
    current grid (no grid is built for it); device=True evaluates func on the
    host per level and computes the nodes on the GPU (mwgpu_project_level_values)."""
    if callable(gaussians):
        return _project_func(prec, tree, gaussians, max_iter, abs_prec, device)
    if grid:
        build_grid(tree, gaussians)
    coef, ex, pos = _gauss_arrays(gaussians)
    if device:
        st = MwhApplyStats()
        _ck(lib().mwh_project_gauss_device(float(prec), tree._h, len(coef), _pd(coef), _pd(ex), _pd(pos), int(max_iter), int(bool(abs_prec)),
                                           C.byref(st)))
        return st.as_dict()
    _ck(lib().mwh_project_gauss(float(prec), tree._h, len(coef), _pd(coef), _pd(ex), _pd(pos), int(max_iter), int(bool(abs_prec))))


def _combine(fn, prec, out, terms, max_iter, abs_prec):
    c = np.ascontiguousarray([float(t[0]) for t in terms], dtype=np.float64)
    hs = (_P * len(terms))(*[t[1]._h for t in terms])
    st = MwhApplyStats()
    _ck(fn(float(prec), out._h, len(terms), _pd(c), hs, int(max_iter), int(bool(abs_prec)), C.byref(st)))
    return st.as_dict()


def add(prec, out, *args, max_iter=-1, abs_prec=False):
    """add(prec, out, a, A, b, B) or add(prec, out, [(c, tree), ...]) (src/treebuilders/add.cpp):
    out = sum of c_j f_j, built adaptively on the GPU; returns the statistics."""
    terms = args[0] if len(args) == 1 else [(args[0], args[1]), (args[2], args[3])]
    return _combine(lib().mwh_add, prec, out, terms, max_iter, abs_prec)


def multiply(prec, out, *args, max_iter=-1, abs_prec=False, use_max_norms=False):
    """multiply(prec, out, c, A, B) or multiply(prec, out, [(c, tree), ...]) (src/treebuilders/multiply.cpp):
    out = product of c_j f_j, built adaptively on the GPU; returns the statistics.
    use_max_norms: the grid from the two inputs' max norms (MultiplicationAdaptor,
    two factors, abs_prec not used), else the wavelet adaptor."""
    terms = args[0] if len(args) == 1 else [(args[0], args[1]), (1.0, args[2])]
    if use_max_norms:
        c = np.ascontiguousarray([float(t[0]) for t in terms], dtype=np.float64)
        hs = (_P * len(terms))(*[t[1]._h for t in terms])
        st = MwhApplyStats()
        _ck(lib().mwh_multiply_max_norms(float(prec), out._h, len(terms), _pd(c), hs, int(max_iter), C.byref(st)))
        return st.as_dict()
    return _combine(lib().mwh_multiply, prec, out, terms, max_iter, abs_prec)


def copy_grid(out, inp):
    _ck(lib().mwh_copy_grid(out._h, inp._h))


def dot(a, b):
    return lib().mwh_dot(a._h, b._h)


class ConvolutionOperator:
    """Separated Gaussian convolution operator (src/operators/ConvolutionOperator.h).

    ConvolutionOperator(mra, kernel, prec) is ConvolutionOperator<3>(MRA, kernel,
    prec) (ConvolutionOperator.cpp:51-62): kernel = (exponents, coefficients) of
    the 1D Gaussians, e.g. from helmholtz_kernel / poisson_kernel."""

    def __init__(self, mra, handle, prec=None):
        if prec is not None:
            ex = np.ascontiguousarray(handle[0], dtype=np.float64)
            co = np.ascontiguousarray(handle[1], dtype=np.float64)
            if ex.shape != co.shape or ex.ndim != 1:
                raise ValueError("kernel: exponents and coefficients of equal length")
            h = _P()
            _ck(lib().mwh_convolution(mra._h, len(ex), _pd(ex), _pd(co), float(prec), C.byref(h)))
            handle = h
            self.prec = prec
        self.mra = mra
        self._h = handle
        nt, nn, nr = C.c_int(), C.c_int(), C.c_int()
        _ck(lib().mwh_oper_info(self._h, C.byref(nt), C.byref(nn), C.byref(nr)))
        self.n_terms, self.n_nodes, self.n_rows = nt.value, nn.value, nr.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mwh_oper_free(self._h)
            self._h = None

    def size(self):
        return self.n_terms

    def export(self):
        """Node caches: depth[T], max_transl[rows], blocks[nodes,4,K,K] (column-major blocks), norms[nodes,4], kernel."""
        K = self.mra.kp1
        depth = np.zeros(self.n_terms, dtype=np.int32)
        mt = np.zeros(self.n_rows, dtype=np.int32)
        blocks = np.zeros(self.n_nodes * 4 * K * K)
        norms = np.zeros(self.n_nodes * 4)
        kexp = np.zeros(self.n_terms)
        kcoef = np.zeros(self.n_terms)
        _ck(lib().mwh_oper_export(self._h, _pi(depth), _pi(mt), _pd(blocks), _pd(norms), _pd(kexp), _pd(kcoef)))
        return {"depth": depth, "max_transl": mt, "blocks": blocks, "norms": norms, "kernel_exp": kexp, "kernel_coef": kcoef}

    def desc(self):
        d = MwgpuOperDesc()
        _ck(lib().mwh_oper_desc(self._h, C.byref(d)))
        return d


class PoissonOperator(ConvolutionOperator):
    """PoissonOperator(MRA, prec): 1/r as a sum of Gaussians (src/operators/PoissonOperator.cpp:40-55)."""

    def __init__(self, mra, prec):
        h = _P()
        _ck(lib().mwh_poisson(mra._h, float(prec), C.byref(h)))
        super().__init__(mra, h)
        self.prec = prec


class HelmholtzOperator(ConvolutionOperator):
    """HelmholtzOperator(MRA, mu, prec): exp(-mu r)/r (src/operators/HelmholtzOperator.cpp:41-56)."""

    def __init__(self, mra, mu, prec):
        h = _P()
        _ck(lib().mwh_helmholtz(mra._h, float(mu), float(prec), C.byref(h)))
        super().__init__(mra, h)
        self.prec = prec
        self.mu = mu


class IdentityConvolution(ConvolutionOperator):
    """IdentityConvolution<3>(MRA, prec) (src/operators/IdentityConvolution.cpp:41-55):
    the kernel is one normalised Gaussian of exponent sqrt(1 / k_prec),
    k_prec = prec / 10 (IdentityKernel.h:34-41), an approximate delta function."""

    def __init__(self, mra, prec):
        expo = float(np.sqrt(10.0 / prec))
        super().__init__(mra, ([expo], [(expo / np.pi) ** 1.5]), prec)


class ABGVOperator(ConvolutionOperator):
    """ABGVOperator(MRA, a, b): first derivative with boundary parameters a, b
    (src/operators/ABGVOperator.cpp:45-71); a = b = 0.5 central difference,
    a = b = 0 center difference."""

    def __init__(self, mra, a, b):
        h = _P()
        _ck(lib().mwh_abgv(mra._h, float(a), float(b), C.byref(h)))
        super().__init__(mra, h)
        self.a, self.b = a, b


class PHOperator(ConvolutionOperator):
    """PHOperator(MRA, order, filter_dir=None): Holoborodko's smoothing
    derivative of order 1 or 2 (src/operators/PHOperator.cpp:40-68); its tables
    are read from the reference's filter files in filter_dir (default: the
    MWFILTERS_DIR environment variable).  Apply with apply(out, D, inp, dir)."""

    def __init__(self, mra, order, filter_dir=None):
        h = _P()
        _ck(lib().mwh_ph(mra._h, int(order), None if filter_dir is None else os.fsencode(filter_dir), C.byref(h)))
        super().__init__(mra, h)
        self.order = order


class BSOperator(ConvolutionOperator):
    """BSOperator(MRA, order, filter_dir=None): the B-spline derivative of order
    1, 2 or 3 (src/operators/BSOperator.cpp:40-68), tables as for PHOperator."""

    def __init__(self, mra, order, filter_dir=None):
        h = _P()
        _ck(lib().mwh_bs(mra._h, int(order), None if filter_dir is None else os.fsencode(filter_dir), C.byref(h)))
        super().__init__(mra, h)
        self.order = order


class TableDerivativeOperator(ConvolutionOperator):
    """A derivative operator of the given order from the three blocks S_+1, S_0,
    S_-1 ((k+1) x (k+1), as PHCalculator / BSCalculator read them)."""

    def __init__(self, mra, order, s_p1, s_0, s_m1):
        K = mra.kp1
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(K, K) for a in (s_p1, s_0, s_m1)]
        h = _P()
        _ck(lib().mwh_deriv_tables(mra._h, int(order), _pd(arrs[0]), _pd(arrs[1]), _pd(arrs[2]), C.byref(h)))
        super().__init__(mra, h)
        self.order = order


def _kernel(fn, *args):
    n = fn(*args, 0, None, None)
    if n < 0:
        _ck(n)
    ex = np.zeros(n)
    co = np.zeros(n)
    fn(*args, n, _pd(ex), _pd(co))
    return ex, co


def poisson_kernel(eps, r_min, r_max):
    """PoissonKernel(eps, r_min, r_max): (exponents, coefficients)."""
    return _kernel(lib().mwh_poisson_kernel, float(eps), float(r_min), float(r_max))


def helmholtz_kernel(mu, eps, r_min, r_max):
    """HelmholtzKernel(mu, eps, r_min, r_max): (exponents, coefficients)."""
    return _kernel(lib().mwh_helmholtz_kernel, float(mu), float(eps), float(r_min), float(r_max))


def apply(*args, **kw):
    """mrcpp::apply on the GPU, returning the apply statistics:
    apply(prec, out, oper, inp, max_iter=-1, abs_prec=False, precision=FP64) for a
    convolution operator; apply(prec, out, oper, inp, prec_trees, max_iter,
    abs_prec, precision=FP64), or prec_trees=[...] as a keyword, for the form
    whose precision is scaled per node by the largest norm of the precision
    trees (src/treebuilders/apply.h:43); apply(out, oper, inp, dir) for a
    derivative operator (ABGVOperator; output grid = input grid widened along
    dir, FP64)."""
    if args and isinstance(args[0], FunctionTree):
        return apply_derivative(*args, **kw)
    return _apply_convolution(*args, **kw)


def _apply_convolution(prec, out, oper, inp, *rest, max_iter=-1, abs_prec=False, precision=FP64, prec_trees=None):
    rest = list(rest)
    if rest and isinstance(rest[0], (list, tuple)):
        prec_trees = rest.pop(0)
    if len(rest) > 3:
        raise TypeError("apply: too many positional arguments")
    vals = dict(zip(["max_iter", "abs_prec", "precision"], rest))
    max_iter = vals.get("max_iter", max_iter)
    abs_prec = vals.get("abs_prec", abs_prec)
    precision = vals.get("precision", precision)
    st = MwhApplyStats()
    if prec_trees is None:
        _ck(lib().mwh_apply(float(prec), out._h, oper._h, inp._h, int(max_iter), int(bool(abs_prec)), int(precision), C.byref(st)))
    else:
        pts = list(prec_trees)
        arr = (_P * max(len(pts), 1))(*[t._h for t in pts])
        _ck(lib().mwh_apply_prec(float(prec), out._h, oper._h, inp._h, len(pts), arr, int(max_iter), int(bool(abs_prec)),
                                 int(precision), C.byref(st)))
    return st.as_dict()


def prec_factors(prec_trees, idx):
    """precFac of the precTrees form of apply (apply.cpp:222-229) for the nodes
    idx[j] = (n, l0, l1, l2): 1 / the largest sqrt(maxSquareNorm) over the trees."""
    idx = np.ascontiguousarray(idx, dtype=np.int32).reshape(-1, 4)
    pts = list(prec_trees)
    arr = (_P * max(len(pts), 1))(*[t._h for t in pts])
    fac = np.zeros(len(idx))
    _ck(lib().mwh_prec_factors(len(pts), arr, len(idx), _pi(idx), _pd(fac)))
    return fac


def pinned_stats():
    """Host memory of tree coefficients: state 1 when blocks of 4 MiB and more
    are page-locked (device copies run as DMA), -1 when declined (no device, or
    MWH_PAGEABLE=1), 0 before the first large tree; with the page-locked bytes
    held by trees and idle in the cache."""
    live, idle = C.c_ulonglong(), C.c_ulonglong()
    state = lib().mwh_pinned_stats(C.byref(live), C.byref(idle))
    return {"state": int(state), "live_bytes": int(live.value), "idle_bytes": int(idle.value)}


def apply_derivative(out, oper, inp, dir):
    """apply(out, DerivativeOperator, inp, dir) (src/treebuilders/apply.cpp:379-412)."""
    st = MwhApplyStats()
    _ck(lib().mwh_apply_derivative(out._h, oper._h, inp._h, int(dir), C.byref(st)))
    return st.as_dict()


def apply_batch(prec, outs, oper, inps, max_iter=-1, abs_prec=False, precision=FP64):
    """outs[t] = oper(inps[t]) for every t: the loop of mrcpp::apply calls over a
    set of functions, computed in lockstep so that every TreeBuilder iteration
    of all functions is one device pass.  Each result equals apply() of its
    pair.  Returns the summed statistics."""
    outs, inps = list(outs), list(inps)
    if len(outs) != len(inps) or not outs:
        raise ValueError("apply_batch needs as many outputs as inputs")
    n = len(outs)
    po = (_P * n)(*[o._h for o in outs])
    pi = (_P * n)(*[i._h for i in inps])
    st = MwhApplyStats()
    _ck(lib().mwh_apply_batch(float(prec), n, po, oper._h, pi, int(max_iter), int(bool(abs_prec)), int(precision), C.byref(st)))
    return st.as_dict()


def _pf(a):
    return a.ctypes.data_as(_PF)


MLP_PARAMS = 4801
MLP_FEATURES = 8
DEFAULT_NETWORK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "grid_mlp_k7.npz")


class GridNetwork:
    """The learned output-grid network (3 layers, 64 wide, BF16 weights): its
    FP32 parameters, W1[64][8], b1, W2[64][64], b2, W3[64], b3."""

    def __init__(self, params):
        self.params = np.ascontiguousarray(np.asarray(params, dtype=np.float32))
        if self.params.shape != (MLP_PARAMS,):
            raise ValueError("expected %d parameters" % MLP_PARAMS)
        h = _P()
        _ck(lib().mwh_mlp_create(_pf(self.params), C.byref(h)))
        self._h = h

    FEATURES = 2  # feature set of include/mwgpu.h (wavelet norm, branch / leaf / absent)

    @classmethod
    def load(cls, path=DEFAULT_NETWORK):
        with np.load(path) as z:
            version = int(z["features"]) if "features" in z.files else 1
            if version != cls.FEATURES:
                raise ValueError("%s was trained on another feature set; retrain it" % path)
            net = cls(z["params"])
            net.meta = {k: z[k] for k in z.files if k != "params"}
        return net

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mwh_mlp_free(self._h)
            self._h = None


def apply_learned(prec, out, oper, inp, network, threshold=0.3, full_levels=0, abs_prec=False, precision=FP64):
    """mrcpp::apply(prec, out, oper, inp) with the output grid proposed by the
    network (the first `full_levels` levels refined without it) and judged on
    the device by the split test: the result equals
    apply(prec, out, oper, inp, precision=precision).  Returns the statistics
    (proposal size, first missed level, further passes, round trips, timings)."""
    st = MwhLearnedStats()
    _ck(lib().mwh_apply_learned(float(prec), out._h, oper._h, inp._h, network._h, float(threshold), int(full_levels), int(bool(abs_prec)),
                                int(precision), C.byref(st)))
    return st.as_dict()


def grid_features(prec, grid, oper, inp):
    """Features of every node of `grid` against inp (rows in the order of
    grid.export()), and labels (1 = the node has children): training data for
    the network."""
    n = grid.n_nodes
    x = np.zeros((n, MLP_FEATURES), dtype=np.float32)
    y = np.zeros(n, dtype=np.float32)
    _ck(lib().mwh_grid_features(float(prec), grid._h, oper._h, inp._h, _pf(x), _pf(y)))
    return x, y
