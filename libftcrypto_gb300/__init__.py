"""libftcrypto_gb300 — libftcrypto's batched additively homomorphic ElGamal
over Ed25519, implemented as hand-written CUDA kernels for NVIDIA GB300
(sm_103a) behind the reference's ftcrypto.h C ABI (libftcrypto.so).

    from libftcrypto_gb300 import Array, encrypt
    a = Array.from_small_scalars([1, 2, 3])
    a.add(a)
    a.to_bytes_folded()

The C library is the product; this package builds it (build.py), binds it
(_lib.py) and mirrors its interface in Python (api.py).
"""
from .api import (AFFINE, DECRYPT_MAX_M, EXTENDED, FOLDED, NO_PLAINTEXT, PACKED, TUNE_BATCH_ADD_PTS,  # noqa: F401
                  TUNE_LADDER_BLOCK, TUNE_SCALE_WINDOW, Array, Batch, FtError, check, decrypt, device_memory, encrypt, encrypt_device,
                  ct_add, ct_scan, ct_segmented_sum_csr_device, ct_sub, error_str, init, rerandomise, rerandomise_device, Server, segmented_sum_csr,
                  segmented_sum_csr_device, stream_handle, synchronize, tune, tune_get)
from .build import LIB as LIB_PATH  # noqa: F401
from .build import build  # noqa: F401
