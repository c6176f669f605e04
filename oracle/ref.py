"""ctypes front end of oracle/_ref/libftref.so: the reference's own
sodium_fe.cu / sodium_ge.cu compiled for the host by oracle/build_ref.sh.

TEST INFRASTRUCTURE ONLY: pins the oracle (tests/test_oracle.py) and
generates tests/golden/ (tests/golden/make_golden.py).  Available only where
the reference source tree was present at build time; callers skip otherwise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import REF_LIB_PATH

_lib = None


def available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(REF_LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        for name, res, args in [
            ("ref_decode", I, [P, P]), ("ref_encode", None, [P, P]),
            ("ref_zero", None, [P]), ("ref_base", None, [P]),
            ("ref_scalarmult", None, [P, P, P]), ("ref_scalarmult_base", None, [P, P]),
            ("ref_addto", None, [P, P]), ("ref_subfrom", None, [P, P]),
            ("ref_neg", None, [P]), ("ref_iszero", I, [P]), ("ref_equal", I, [P, P]),
            ("ref_valid", I, [P]), ("ref_to_affine", None, [P, P]),
            ("ref_from_affine", None, [P, P]), ("ref_base_table_entry", None, [P, I, I]),
            ("ref_fe_tobytes", None, [P, P]), ("ref_fe_frombytes", None, [P, P]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _buf(b: bytes | np.ndarray, size: int):
    return ctypes.create_string_buffer(bytes(b), size)


class Pt:
    """One reference ge25519_p3 (160 bytes of 10 x int32 limbs per coord)."""

    def __init__(self, raw: bytes | None = None):
        self.b = ctypes.create_string_buffer(raw if raw is not None else b"\0" * 160, 160)

    def raw(self) -> bytes:
        return self.b.raw

    def copy(self) -> "Pt":
        return Pt(self.b.raw)

    def enc(self) -> bytes:
        out = ctypes.create_string_buffer(32)
        lib().ref_encode(out, self.b)
        return out.raw


def decode(enc: bytes):
    p = Pt()
    r = lib().ref_decode(p.b, _buf(enc, 32))
    return p, r


def zero() -> Pt:
    p = Pt()
    lib().ref_zero(p.b)
    return p


def base() -> Pt:
    p = Pt()
    lib().ref_base(p.b)
    return p


def scalarmult(s: bytes, p: Pt) -> Pt:
    h = Pt()
    lib().ref_scalarmult(h.b, _buf(s, 32), p.b)
    return h


def scalarmult_base(s: bytes) -> Pt:
    h = Pt()
    lib().ref_scalarmult_base(h.b, _buf(s, 32))
    return h


def addto(dest: Pt, src: Pt) -> None:
    lib().ref_addto(dest.b, src.b)


def subfrom(dest: Pt, src: Pt) -> None:
    lib().ref_subfrom(dest.b, src.b)


def neg(p: Pt) -> None:
    lib().ref_neg(p.b)


def iszero(p: Pt) -> int:
    return lib().ref_iszero(p.b)


def equal(a: Pt, b: Pt) -> int:
    return lib().ref_equal(a.b, b.b)


def valid(p: Pt) -> int:
    return lib().ref_valid(p.b)


def to_affine(p: Pt) -> bytes:
    out = ctypes.create_string_buffer(64)
    lib().ref_to_affine(out, p.b)
    return out.raw


def from_affine(aff: bytes) -> Pt:
    p = Pt()
    lib().ref_from_affine(p.b, _buf(aff, 64))
    return p


def base_table_entry(i: int, j: int) -> bytes:
    out = ctypes.create_string_buffer(96)
    lib().ref_base_table_entry(out, i, j)
    return out.raw
