"""ctypes front end of the CPU oracle (oracle/ftoracle.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / --impl reference legs as the checker; the shipped
library (libftcrypto_gb300) never imports it.

Point arrays are numpy uint8 arrays of shape (n, 128) in the packed128 layout
(X, Y, Z, T as 32-byte little-endian integers congruent mod 2^255-19).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libftoracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libftref.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile oracle/ftoracle.c into oracle/libftoracle.so with gcc."""
    src = os.path.join(HERE, "ftoracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(
            ["gcc", "-O3", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lpthread"])
    return LIB_PATH


def build_ref() -> str | None:
    """Build oracle/_ref/libftref.so from the reference sources, if present
    (the recipe oracle/build_ref.sh knows where they lie)."""
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return REF_LIB_PATH if os.path.exists(REF_LIB_PATH) else None


def ref_src() -> str:
    """The reference's src/ directory as oracle/build_ref.sh resolves it
    (FT_REF_SRC, else its default); it may not exist."""
    return subprocess.check_output(["sh", os.path.join(HERE, "build_ref.sh"), "--src"], text=True).strip()


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        S = ctypes.c_size_t
        I = ctypes.c_int
        sig = {
            "fto_init": (I, []),
            "fto_encode": (None, [P, P, S]),
            "fto_encode_mt": (None, [P, P, S, I]),
            "fto_decode": (ctypes.c_int64, [P, P, S]),
            "fto_to_affine": (None, [P, P, S]),
            "fto_from_affine": (None, [P, P, S]),
            "fto_to_ref160": (None, [P, P, S]),
            "fto_from_ref160": (None, [P, P, S]),
            "fto_set_zero": (None, [P, S]),
            "fto_from_scalars": (None, [P, P, S, I]),
            "fto_from_scalars_comb": (None, [P, P, S, I]),
            "fto_add": (None, [P, P, S, I]),
            "fto_sub": (None, [P, P, S, I]),
            "fto_neg": (None, [P, S]),
            "fto_mul": (None, [P, P, S, I]),
            "fto_scale": (None, [P, P, S, I]),
            "fto_scale_u64": (None, [P, ctypes.c_uint64, S, I]),
            "fto_scale_u64_each": (None, [P, P, S, I]),
            "fto_index": (None, [P, P, S]),
            "fto_equal": (None, [P, P, P, S]),
            "fto_validate": (ctypes.c_int64, [P, S]),
            "fto_reduce": (None, [P, P, S, I]),
            "fto_scan": (None, [P, S, I]),
            "fto_scan_mt": (None, [P, S, I, I]),
            "fto_segsum_csr": (None, [P, P, S, P, I]),
            "fto_isum": (I, [P, S, P, S, P]),
            "fto_encrypt": (I, [P, P, P, P, P, S, I]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L.fto_init()
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def _pts(n):
    return np.zeros((n, 128), dtype=np.uint8)


def encode(pts: np.ndarray, threads: int = 1) -> np.ndarray:
    """Canonical encodings; threads > 1 uses the batched-inversion form
    (fto_encode_mt), which gives the same bytes."""
    pts = np.ascontiguousarray(pts)
    n = pts.shape[0]
    out = np.zeros((n, 32), dtype=np.uint8)
    if threads > 1:
        lib().fto_encode_mt(_p(out), _p(pts), n, threads)
    else:
        lib().fto_encode(_p(out), _p(pts), n)
    return out


def decode(enc: np.ndarray):
    n = enc.shape[0]
    pts = _pts(n)
    bad = lib().fto_decode(_p(pts), _p(np.ascontiguousarray(enc)), n)
    return pts, int(bad)


def to_affine(pts):
    out = np.zeros((pts.shape[0], 64), dtype=np.uint8)
    lib().fto_to_affine(_p(out), _p(pts), pts.shape[0])
    return out


def from_affine(aff):
    pts = _pts(aff.shape[0])
    lib().fto_from_affine(_p(pts), _p(np.ascontiguousarray(aff)), aff.shape[0])
    return pts


def to_ref160(pts):
    out = np.zeros((pts.shape[0], 160), dtype=np.uint8)
    lib().fto_to_ref160(_p(out), _p(pts), pts.shape[0])
    return out


def from_ref160(raw):
    pts = _pts(raw.shape[0])
    lib().fto_from_ref160(_p(pts), _p(np.ascontiguousarray(raw)), raw.shape[0])
    return pts


def zeros(n):
    pts = _pts(n)
    lib().fto_set_zero(_p(pts), n)
    return pts


def from_scalars(scalars: np.ndarray, threads: int = 1, comb: bool = False):
    n = scalars.shape[0]
    pts = _pts(n)
    f = lib().fto_from_scalars_comb if comb else lib().fto_from_scalars
    f(_p(pts), _p(np.ascontiguousarray(scalars)), n, threads)
    return pts


def small_to_scalars(m) -> np.ndarray:
    m = np.ascontiguousarray(np.asarray(m, dtype=np.uint64))
    out = np.zeros((m.shape[0], 32), dtype=np.uint8)
    out[:, :8] = m.view(np.uint8).reshape(-1, 8)
    return out


def add(a, b, threads=1):
    r = a.copy()
    lib().fto_add(_p(r), _p(b), a.shape[0], threads)
    return r


def sub(a, b, threads=1):
    r = a.copy()
    lib().fto_sub(_p(r), _p(b), a.shape[0], threads)
    return r


def neg(a):
    r = a.copy()
    lib().fto_neg(_p(r), a.shape[0])
    return r


def mul(a, scalars, threads=1):
    r = a.copy()
    lib().fto_mul(_p(r), _p(np.ascontiguousarray(scalars)), a.shape[0], threads)
    return r


def scale(a, scalar, threads=1):
    r = a.copy()
    s = np.ascontiguousarray(np.asarray(scalar, dtype=np.uint8).reshape(32))
    lib().fto_scale(_p(r), _p(s), a.shape[0], threads)
    return r


def scale_u64(a, k: int, threads=1):
    """k * a_i for a public k < 2^64 by double-and-add: the group element of
    scale(a, k) (canonical encodings equal on the curve)."""
    r = np.ascontiguousarray(a).copy()
    lib().fto_scale_u64(_p(r), int(k), r.shape[0], threads)
    return r


def scale_u64_each(a, ks, threads=1):
    """k_i * a_i for public k_i < 2^64, one per point, by double-and-add."""
    r = np.ascontiguousarray(a).copy()
    kk = np.ascontiguousarray(np.asarray(ks, dtype=np.uint64))
    assert kk.shape[0] == r.shape[0]
    lib().fto_scale_u64_each(_p(r), _p(kk), r.shape[0], threads)
    return r


def index(a):
    out = np.zeros(a.shape[0], dtype=np.int64)
    lib().fto_index(_p(out), _p(a), a.shape[0])
    return out


def equal(a, b):
    out = np.zeros(a.shape[0], dtype=np.int64)
    lib().fto_equal(_p(out), _p(a), _p(b), a.shape[0])
    return out


def validate(a) -> int:
    return int(lib().fto_validate(_p(a), a.shape[0]))


def reduce(a, threads=1):
    out = _pts(1)
    lib().fto_reduce(_p(out), _p(a), a.shape[0], threads)
    return out


def scan(a, exclusive=False, threads=1):
    """Prefix sums; threads > 1 scans chunks in parallel (same group
    elements, other projective coordinates: compare encodings)."""
    r = np.ascontiguousarray(a).copy()
    if threads > 1:
        lib().fto_scan_mt(_p(r), r.shape[0], 1 if exclusive else 0, threads)
    else:
        lib().fto_scan(_p(r), r.shape[0], 1 if exclusive else 0)
    return r


def segsum_csr(offsets, src, threads=1):
    off = np.ascontiguousarray(np.asarray(offsets, dtype=np.int32))
    nseg = off.shape[0] - 1
    out = _pts(nseg)
    lib().fto_segsum_csr(_p(out), _p(off), nseg, _p(src), threads)
    return out


def isum(res, idxs, src):
    r = res.copy()
    ix = np.ascontiguousarray(np.asarray(idxs, dtype=np.uint64))
    err = lib().fto_isum(_p(r), r.shape[0], _p(ix), ix.shape[0], _p(src))
    return r, int(err)


def encrypt(pk32, m, r, threads=1):
    n = len(m)
    c1, c2 = _pts(n), _pts(n)
    mm = np.ascontiguousarray(np.asarray(m, dtype=np.uint64))
    pk = np.ascontiguousarray(np.asarray(pk32, dtype=np.uint8).reshape(32))
    err = lib().fto_encrypt(_p(c1), _p(c2), _p(pk), _p(mm), _p(np.ascontiguousarray(r)), n, threads)
    if err:
        raise ValueError("invalid public key")
    return c1, c2
