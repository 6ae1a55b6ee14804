"""ctypes binding of libtreecode.so (the C ABI in include/treecode.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when the shared object has not been built (``python -m
masterthesislucas_gb300.build`` or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtreecode.so")

TC_OK = 0
TC_ERR_INVALID = -1
TC_ERR_CUDA = -2
TC_ERR_NOMEM = -3
TC_ERR_STATE = -4
TC_ERR_TIMEOUT = -5

TC_KERNEL_TSNE = 0
TC_KERNEL_GRAVITY = 1
TC_PREC_FP32 = 0
TC_PREC_FP64 = 1
TC_VARIANT_SYM = 0
TC_VARIANT_MORTON = 1
TC_MAC_CELL = 0
TC_REPULSION_TREE = 0
TC_REPULSION_PM = 1
TC_MAC_BMAX = 1
TC_CENTRE_COM = 0
TC_CENTRE_BOX = 1
TC_M2L_SIMT = 0
TC_M2L_TENSOR = 1
TC_M2L_TENSOR_ALL = 2


class TcConfig(ctypes.Structure):
    _fields_ = [("kernel", ctypes.c_int), ("max_children", ctypes.c_int), ("depth", ctypes.c_int),
                ("theta", ctypes.c_double), ("softening", ctypes.c_double), ("precision", ctypes.c_int),
                ("device", ctypes.c_int), ("stream", ctypes.c_void_p), ("order", ctypes.c_int)]


class TreecodeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"treecode error {code}: {msg}")
        self.code = code


# every symbol include/treecode.h declares, with its ctypes signature
_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
SIGNATURES = {
    "tc_config_init": (_I, [_P]),
    "tc_create": (_I, [_P, _P]),
    "tc_destroy": (_I, [_P]),
    "tc_set_theta": (_I, [_P, _D]),
    "tc_set_variant": (_I, [_P, _I]),
    "tc_set_mac": (_I, [_P, _I]),
    "tc_set_expansion_centre": (_I, [_P, _I]),
    "tc_knn_device": (_I, [_P, _I64, _I, _I, _P, _P, _P]),
    "tc_perplexity_device": (_I, [_P, _I64, _I, ctypes.c_double, _I, ctypes.c_double, _P, _P]),
    "tc_symmetrize_device": (_I, [_P, _P, _I64, _I, _P, _P, _P, _P, _P]),
    "tc_set_m2l_engine": (_I, [_P, _I]),
    "tc_set_near_overlap": (_I, [_P, _I]),
    "tc_set_adaptive_order": (_I, [_P, _D]),
    "tc_set_leaf_p2p": (_I, [_P, _I]),
    "tc_pm_solve": (_I, [_I, _D, _I, _P, _I64, _P, _P]),
    "tc_tsne_set_repulsion": (_I, [_P, _I, _D]),
    "tc_pm_solve_device": (_I, [_I, _D, _I, _P, _I64, _P, _P, _P]),
    "tc_get_depth": (_I, [_I, _I64, _P]),
    "tc_node_count": (_I, [ctypes.c_uint32, _P]),
    "tc_update_tree": (_I, [_P, _P, _P, _I64, _P, _P]),
    "tc_solve": (_I, [_P, _P, _P, _P, _I64]),
    "tc_update_tree_device": (_I, [_P, _P, _I64, _P, _P]),
    "tc_solve_device": (_I, [_P, _P, _P, _I, _I]),
    "tc_get_tree": (_I, [_P, _P, _P, _P, _P]),
    "tc_get_list_stats": (_I, [_P, _P, _P]),
    "tc_get_node_boxes": (_I, [_P, _I, _P, _I64, _P]),
    "tc_last_launch_count": (_I, [_P]),
    "tc_get_stage_times": (_I, [_P, _P]),
    "tc_get_counters": (_I, [_P, _P]),
    "tc_last_error": (ctypes.c_char_p, []),
    "tc_direct": (_I, [_I, _D, _I, _P, _I64, _P, _I64, _P, _P]),
    "tc_direct_device": (_I, [_I, _D, _I, _P, _I64, _P, _I64, _P, _P, _P]),
    "tc_direct_device_noalloc": (_I, [_I, _D, _I, _P, _I64, _P, _I64, _P, _P, _P]),
    "tc_bh_solve": (_I, [_I, _D, _I, _D, _I, _P, _I64, _P, _P]),
    "tc_bh_solve_device": (_I, [_I, _D, _I, _D, _I, _P, _I64, _P, _P, _P]),
    "tc_bhmp_solve": (_I, [_I, _D, _I, _D, _I, _P, _I64, _P, _P]),
    "tc_bhmp_solve_device": (_I, [_I, _D, _I, _D, _I, _P, _I64, _P, _P, _P]),
    "tc_mlp_create": (_I, [ctypes.c_uint64, _P]),
    "tc_mlp_destroy": (_I, [_P]),
    "tc_mlp_set_normalization": (_I, [_P, _P, _P]),
    "tc_mlp_get_params": (_I, [_P, _P, _P, _P]),
    "tc_mlp_set_params": (_I, [_P, _P]),
    "tc_mlp_gradient": (_I, [_P, _P, _P, _I64, _P, _P]),
    "tc_mlp_train": (_I, [_P, _P, _P, _I64, _I, _I, ctypes.c_float, ctypes.c_uint64, _P]),
    "tc_mlp_forward": (_I, [_P, _P, _I64, _P]),
    "tc_mlp_forward_tc": (_I, [_P, _P, _I64, _P]),
    "tc_lc_pair_errors": (_I, [_P, _P, _I64, _P, _P]),
    "tc_get_list": (_I, [_P, _I, _I, _P, _P, _P]),
    "tc_set_controller": (_I, [_P, _P, ctypes.c_double]),
    "tc_leapfrog_step": (_I, [_P, _P, _P, _P, _I64, _D, _D, _I, _P]),
    "tc_tsne_create": (_I, [_P, _I64, _P, _P, _P, _P, _P]),
    "tc_tsne_destroy": (_I, [_P]),
    "tc_tsne_set_theta": (_I, [_P, _D]),
    "tc_tsne_set_depth": (_I, [_P, _I]),
    "tc_tsne_step": (_I, [_P, _D, _D, _D, _P]),
    "tc_tsne_get": (_I, [_P, _P, _P, _P]),
    "tc_tsne_last_launch_count": (_I, [_P]),
    "tc_tsne_batch_create": (_I, [_P, _I, _D, _P]),
    "tc_tsne_batch_destroy": (_I, [_P]),
    "tc_tsne_batch_step": (_I, [_P, _D, _D, _D]),
    "tc_tsne_batch_stats": (_I, [_P, _P]),
    "tc_tsne_batch_set_capture": (_I, [_P, _I]),
    "tc_async_status": (_I, [_P]),
    "tc_step_capture": (_I, [_P, _P, _I64, _P, _P, _P, _I]),
    "tc_step_launch": (_I, [_P]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                               "(the CUDA library is required; there is no CPU path)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != TC_OK:
        msg = lib().tc_last_error()
        raise TreecodeError(rc, msg.decode() if msg else "")
    return rc


def ptr(a):
    """ctypes pointer of a numpy array (host) or a torch tensor (device); None passes NULL."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)
