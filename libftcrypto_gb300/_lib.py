"""ctypes binding of libftcrypto.so (include/ftcrypto.h + include/ftcrypto_gb300.h).

Loading fails loudly when the compiled library is missing: there is no
fallback implementation.  This module is also the binding a Python caller
of the reference library would write against the same header.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libftcrypto.so")

P = ctypes.c_void_p
S = ctypes.c_size_t
I = ctypes.c_int
U = ctypes.c_uint
PP = ctypes.POINTER(ctypes.c_void_p)
PS = ctypes.POINTER(ctypes.c_size_t)
PI64 = ctypes.POINTER(ctypes.c_int64)

# name: (restype, argtypes) — in the order of include/ftcrypto.h
SIGNATURES = {
    "ft_error_str": (ctypes.c_char_p, [I]),
    "ft_crypto_init": (I, []),
    "ft_crypto_device_memory": (I, [PS, PS]),
    "ft_array_init_scalar": (I, [PP, S, P]),
    "ft_array_init_point": (I, [PP, S, P, S]),
    "ft_array_get_subset": (I, [PP, P, S, P]),
    "ft_array_get_range": (I, [PP, S, S, S, P]),
    "ft_array_assign_to_subset": (I, [P, P, S, P]),
    "ft_array_assign_zero_to_subset": (I, [P, P, S]),
    "ft_array_assign_to_range": (I, [P, S, S, S, P]),
    "ft_array_delete_subset": (I, [P, P, S]),
    "ft_array_delete_range": (I, [P, S, S, S]),
    "ft_array_to_bytes_folded": (I, [P, S, P]),
    "ft_array_to_bytes_affine": (I, [P, S, P]),
    "ft_array_to_bytes": (I, [P, S, P]),
    "ft_array_from_bytes_folded": (I, [PI64, PP, P, S]),
    "ft_array_from_bytes_affine": (I, [PP, P, S]),
    "ft_array_from_bytes": (I, [PP, P, S]),
    "ft_array_validate": (I, [PI64, P]),
    "ft_array_from_scalars": (I, [PP, P, S]),
    "ft_array_from_small_scalars": (I, [PP, P, S]),
    "ft_array_free": (None, [P]),
    "ft_array_get_length": (S, [P]),
    "ft_array_set_length": (I, [P, S]),
    "ft_array_mux": (I, [P, P, P]),
    "ft_array_contains": (I, [P, P, P]),
    "ft_add": (I, [P, P]),
    "ft_reduce_isum": (I, [P, P, S, P]),
    "ft_sub": (I, [P, P]),
    "ft_scale": (None, [P, P]),
    "ft_neg": (None, [P]),
    "ft_mul": (I, [P, P, S]),
    "ft_index": (None, [P, P]),
    "ft_equal": (I, [P, P, P]),
    "ft_not_equal": (I, [P, P, P]),
    "ft_array_prescan": (I, [P]),
    "ft_array_scan": (I, [P]),
    "ft_array_reduce": (I, [P]),
    # extensions (ftcrypto_gb300.h)
    "ftx_last_error": (I, []),
    "ftx_last_cuda_error": (I, []),
    "ftx_stream": (P, []),
    "ftx_synchronize": (I, []),
    "ftx_array_device_view": (I, [P, PP, PS]),
    "ftx_array_to_packed": (I, [P, S, P]),
    "ftx_array_from_packed": (I, [PP, P, S]),
    "ftx_mul_device": (I, [P, P, S]),
    "ftx_encrypt": (I, [PP, PP, P, P, P, S, U]),
    "ftx_encrypt_device": (I, [P, P, P, P, P, S, U]),
    "ftx_ct_add": (I, [P, P, P, P]),
    "ftx_ct_scan": (I, [P, P, I]),
    "ftx_ct_sub": (I, [P, P, P, P]),
    "ftx_rerandomise": (I, [P, P, P, P, S]),
    "ftx_rerandomise_device": (I, [P, P, P, P, S]),
    "ftx_decrypt": (I, [P, P, P, ctypes.c_uint64, P]),
    "ftx_segmented_sum_csr": (I, [PP, P, S, P]),
    "ftx_segmented_sum_csr_device": (I, [P, P, S, P]),
    "ftx_ct_segmented_sum_csr_device": (I, [P, P, P, S, P, P]),
    "ftx_reduce_into": (I, [P, S, P]),
    "ftx_scale_small": (I, [P, ctypes.c_uint32]),
    "ftx_scale_bounded": (I, [P, ctypes.c_uint32, U]),
    "ftx_batch_create": (I, [PP]),
    "ftx_batch_add": (I, [P, P, P]),
    "ftx_batch_scale_small": (I, [P, P, ctypes.c_uint32]),
    "ftx_batch_scale_bounded": (I, [P, P, ctypes.c_uint32, U]),
    "ftx_batch_segmented_sum": (I, [P, P, P, S, P]),
    "ftx_batch_run": (I, [P]),
    "ftx_batch_info": (I, [P, PS, PS]),
    "ftx_batch_free": (None, [P]),
    "ftx_tune": (I, [I, I]),
    "ftx_tune_get": (I, [I]),
    "ftx_scan_noalloc": (I, [P, S, S, I, P]),
}

class Request(ctypes.Structure):
    """ftx_request of include/ftcrypto_gb300.h"""
    _fields_ = [("op", ctypes.c_int), ("n", ctypes.c_size_t), ("m", ctypes.c_void_p),
                ("plaintext_bits", ctypes.c_uint), ("r", ctypes.c_void_p), ("k", ctypes.c_void_p),
                ("offsets", ctypes.c_void_p), ("nseg", ctypes.c_size_t), ("c1", ctypes.c_void_p),
                ("c2", ctypes.c_void_p)]


class Result(ctypes.Structure):
    """ftx_result of include/ftcrypto_gb300.h"""
    _fields_ = [("err", ctypes.c_int), ("c1", ctypes.c_void_p), ("c2", ctypes.c_void_p),
                ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


SIGNATURES.update({
    "ftx_server_create": (I, [PP, P, S, I]),
    "ftx_server_submit": (I, [P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "ftx_server_wait": (I, [P, ctypes.c_uint64, ctypes.POINTER(Result)]),
    "ftx_server_release": (I, [P, P]),
    "ftx_server_stats": (I, [P, PS, PS, PS]),
    "ftx_server_free": (None, [P]),
})

REFERENCE_SYMBOLS = [k for k in SIGNATURES if k.startswith("ft_")]

_lib = None


def load(path: str = LIB_PATH):
    """Load libftcrypto.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m libftcrypto_gb300.build` "
            "(the CUDA library is required; there is no CPU implementation)")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L
