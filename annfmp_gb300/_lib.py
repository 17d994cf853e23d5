"""ctypes binding of libannf_gb300.so (the C ABI in include/annf_gb300.h).

The library is the product's only compute path: every function here raises if the shared
library is missing or a call fails. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libannf_gb300.so")

ANNF_OK = 0
ANNF_ERR_INVALID = -1
ANNF_ERR_UNSUPPORTED = -2
ANNF_ERR_CUDA = -3
ANNF_ERR_ALLOC = -4
ANNF_ERR_STATE = -5
ANNF_ERR_DEVICE = -6
ANNF_ERR_SOLVER = -7

ANNF_OPT_INT_PROJECTION = 1
ANNF_REAL_F32 = 0
ANNF_REAL_F64 = 1
ANNF_SPLIT_CYCLIC = 0
ANNF_SPLIT_LONGEST = 1
ANNF_LEAF_EXACT = 0
ANNF_LEAF_BF16 = 1
ANNF_LEAF_FP16 = 2
ANNF_LEAF_FP8 = 3


class AnnfError(RuntimeError):
    """A failed call into the CUDA library; ``status`` is the ANNF_ERR_* code."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"annf status {status}: {msg}")
        self.status = status


class AnnfUnsupported(AnnfError, NotImplementedError):
    pass


class AnnfInvalid(AnnfError, ValueError):
    pass


class TreeView(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int), ("d", ctypes.c_int), ("depth", ctypes.c_int), ("real_type", ctypes.c_int),
        ("n_leaves", ctypes.c_int),
        ("points", ctypes.c_void_p), ("perm", ctypes.c_void_p), ("node_axis", ctypes.c_void_p),
        ("node_split", ctypes.c_void_p), ("leaf_begin", ctypes.c_void_p), ("point_leaf", ctypes.c_void_p),
        ("leaf_box", ctypes.c_void_p),
    ]


class OclTreeView(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int), ("d", ctypes.c_int), ("height", ctypes.c_int), ("n_nodes", ctypes.c_int),
        ("points_per_leaf", ctypes.c_int), ("m_padded", ctypes.c_int),
        ("points", ctypes.c_void_p), ("indir", ctypes.c_void_p), ("node_dim", ctypes.c_void_p),
        ("node_val", ctypes.c_void_p), ("node_same_dim_ancestor", ctypes.c_void_p), ("orig2leaf", ctypes.c_void_p),
    ]


# every exported symbol and its signature: (restype, argtypes)
_vp, _i, _ll, _u = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_uint
SIGNATURES = {
    "annf_version": (_i, []),
    "annf_last_error": (ctypes.c_char_p, []),
    "annf_create": (_i, [ctypes.POINTER(_vp), _i]),
    "annf_destroy": (None, [_vp]),
    "annf_build_tree": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "annf_tree_get": (_i, [_vp, ctypes.POINTER(TreeView)]),
    "annf_kneighbors": (_i, [_vp, _vp, _i, _i, _ll, _vp, _vp, _vp]),
    "annf_kneighbors_noalloc": (_i, [_vp, _vp, _i, _i, _ll, _vp, _vp, _vp]),
    "annf_process_rows": (_i, [_vp, _vp, _vp, _i, _vp, _i, _i, _vp, _i, _i, _i, _i, _i, _ll, _vp, _vp, _vp]),
    "annf_process_rows_img": (_i, [_vp, _vp, _vp, _i, _i, _vp, _i, _i, _i, _i, _vp, _i, _i, _i, _i, _i, _ll,
                                   _vp, _vp, _vp]),
    "annf_pca_fit": (_i, [_vp, _vp, _i, _i, _vp, _i, _vp, _i, _i, _vp, _i, _i, _i, _i, _vp, _vp, _vp]),
    "annf_pca_fit_subspace": (_i, [_vp, _vp, _i, _i, _vp, _i, _vp, _i, _i, _vp, _i, _i, _i, _i, _i, _vp, _vp, _vp]),
    "annf_project": (_i, [_vp, _vp, _i, _i, _i, _i, _vp, _vp, _i, _i, _vp, _vp]),
    "annf_device_status": (_i, [_vp, _vp, ctypes.POINTER(_u)]),
    "annf_set_option": (_i, [_vp, _i, _i]),
    "annf_ocl_build_tree": (_i, [_vp, _vp, _i, _i, _i, _vp]),
    "annf_ocl_tree_get": (_i, [_vp, ctypes.POINTER(OclTreeView)]),
    "annf_ocl_rows": (_i, [_vp, _vp, _vp, _i, _i, _vp, _i, _i, _i, _i, _vp, _i, _i, _vp, _vp, _vp, _vp]),
    "annf_parallel_nnf": (_i, [_vp, _vp, _vp, _i, _i, _vp, _i, _i, _i, _i, _vp, _i, _vp, _i, _i, _u, _i, _i, _i, _vp,
                               _vp]),
    "annf_parallel_nnf_seeded": (_i, [_vp, _vp, _vp, _i, _i, _vp, _i, _i, _i, _i, _vp, _i, _vp, _i, _u, _i, _i, _i,
                                      _vp, _vp]),
    "annf_seed_matches": (_i, [_vp, _vp, _i, _i, _vp, _i, _i, _i, _i, _vp, _i, _vp, _vp]),
    "annf_tc_tile": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp]),
    "annf_natural_knn": (_i, [_vp, _vp, ctypes.c_longlong, _i, _i, _vp, _vp]),
    "annf_project_f16": (_i, [_vp, _vp, _i, _i, _i, _i, _vp, _vp, _i, _vp, _vp]),
    "annf_cnn_input": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp]),
    "annf_cnn_prep_weights": (_i, [_vp, _vp, _i, _i, _vp, _vp, _vp]),
    "annf_cnn_conv_forward": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp, _vp, _i, _vp, _vp]),
    "annf_cnn_prep_weights_tc": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "annf_cnn_conv_forward_tc": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp, _vp, _i, _vp, _vp]),
    "annf_cnn_conv_backward_data": (_i, [_vp, _vp, _vp, _i, _i, _i, _i, _i, _vp, _vp, _vp]),
    "annf_cnn_conv_backward_weights": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _i, _vp, _vp, _vp]),
    "annf_cnn_wta_loss": (_i, [_vp, _vp, _vp, _vp, ctypes.c_longlong, ctypes.c_float, _vp, _vp, _vp]),
    "annf_cnn_adam": (_i, [_vp, _vp, _vp, _vp, _vp, _i, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                           ctypes.c_float, _i, _vp]),
    "annf_cnn_targets": (_i, [_vp, _vp, _i, _i, _i, _i, _vp, _vp, _vp]),
    "annf_cnn_proposals": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _i, _i, _vp, _vp]),
    "annf_cnn_proposals_per_pixel": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _i, _i, _i, _vp, _vp]),
    "annf_raw_nn": (_i, [_vp, _vp, _i, _i, _vp, _i, _i, _i, _i, _vp, _i, _vp, _vp]),
    "annf_profile_enable": (_i, [_vp, _i]),
    "annf_profile_read": (_i, [_vp, _vp, _i, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_char_p)]),
    "annf_launch_count": (_ll, []),
    "annf_buffer_epoch": (_ll, []),
    "annf_pca_covariance": (_i, [_vp, _vp, _i, _i, _vp, _i, _vp, _i, _i, _vp, _i, _i, _i, _vp, _vp]),
    "annf_pca_components": (_i, [_vp, _i, _i, _i, _vp, _vp]),
}

_lock = threading.Lock()
_lib = None


def load(path: str | None = None):
    """Load (once) and return the ctypes library object. Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(f"{p} is missing: build it with `python -m annfmp_gb300.build` "
                              "(the GPU path has no fallback)")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def launch_count() -> int:
    """Kernels launched by libannf_gb300.so in this process so far."""
    return int(load().annf_launch_count())


def buffer_epoch() -> int:
    """Reallocations of the library's device scratch buffers in this process so far (a captured
    graph is valid while this is unchanged)."""
    return int(load().annf_buffer_epoch())


def check(status: int) -> None:
    if status == ANNF_OK:
        return
    msg = load().annf_last_error().decode(errors="replace")
    if status == ANNF_ERR_UNSUPPORTED:
        raise AnnfUnsupported(status, msg)
    if status == ANNF_ERR_INVALID:
        raise AnnfInvalid(status, msg)
    raise AnnfError(status, msg)


class Handle:
    """Owns one annf_handle (device tree + scratch) on one CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.annf_create(ctypes.byref(h), int(device)))
        self.h = h
        self.device = int(device)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.annf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name: str, *args) -> None:
        check(getattr(self.lib, name)(self.h, *args))

    def profile(self, on: bool) -> None:
        check(self.lib.annf_profile_enable(self.h, int(bool(on))))

    def profile_read(self, stream: int) -> list:
        """[(stage, ms), ...] since the last read (synchronises the stream)."""
        cap = 64
        ms = (ctypes.c_float * cap)()
        names = (ctypes.c_char_p * cap)()
        n = self.lib.annf_profile_read(self.h, stream, cap, ms, names)
        if n < 0:
            check(n)
        return [(names[i].decode(), float(ms[i])) for i in range(n)]

    def tree_view(self) -> TreeView:
        tv = TreeView()
        check(self.lib.annf_tree_get(self.h, ctypes.byref(tv)))
        return tv
