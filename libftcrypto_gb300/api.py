"""Python mirror of the ftcrypto.h interface over libftcrypto.so.

`Array` wraps an ft_ge25519_array handle; each method calls the C function of
the same name in the reference interface (ft_add -> Array.add,
ft_array_scan -> Array.scan, ...), with the same argument meaning, and raises
FtError carrying the reference's error code and string where the C call
returns one.  Host data are numpy arrays: scalars (n, 32) uint8, folded
encodings (n, 32) uint8, affine (n, 64), reference limbs (n, 160),
packed (n, 128).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

FOLDED = 32
AFFINE = 64
EXTENDED = 160
PACKED = 128


class FtError(RuntimeError):
    def __init__(self, code: int):
        self.code = int(code)
        msg = f"ft_error {self.code}: {error_str(self.code)}"
        if self.code in (1, 9):  # out of memory, internal: name the CUDA error behind it
            msg += f" (cudaError {lib().ftx_last_cuda_error()})"
        super().__init__(msg)


def lib():
    return _lib.load()


def error_str(code: int) -> str:
    return lib().ft_error_str(int(code)).decode()


def check(code: int) -> None:
    if code:
        raise FtError(code)


def init() -> None:
    check(lib().ft_crypto_init())


def device_memory():
    f, t = ctypes.c_size_t(), ctypes.c_size_t()
    check(lib().ft_crypto_device_memory(ctypes.byref(f), ctypes.byref(t)))
    return f.value, t.value


def synchronize() -> None:
    check(lib().ftx_synchronize())


def stream_handle() -> int:
    return lib().ftx_stream() or 0


def _buf(a: np.ndarray, dtype, width=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
    if width is not None:
        a = a.reshape(-1, width)
    return a


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _sz(idxs):
    return _buf(idxs, np.uint64)


class Array:
    """An ft_ge25519_array: a device-resident array of Ed25519 points."""

    __slots__ = ("_h",)

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.ft_array_free(h)
            self._h = None

    def free(self) -> None:
        if self._h:
            lib().ft_array_free(self._h)
            self._h = None

    def __len__(self) -> int:
        return int(lib().ft_array_get_length(self._h))

    # ---------------------------------------------------------- constructors
    @staticmethod
    def _new(fn, *args) -> "Array":
        h = ctypes.c_void_p()
        check(fn(ctypes.byref(h), *args))
        return Array(h)

    @classmethod
    def init_scalar(cls, n: int, scalar=None) -> "Array":
        s = None if scalar is None else _ptr(_buf(scalar, np.uint8).reshape(32))
        if scalar is not None:
            sb = _buf(scalar, np.uint8).reshape(32)
            return cls._new(lib().ft_array_init_scalar, n, _ptr(sb))
        return cls._new(lib().ft_array_init_scalar, n, s)

    @classmethod
    def init_point(cls, n: int, src: "Array", idx: int) -> "Array":
        return cls._new(lib().ft_array_init_point, n, src._h, idx)

    @classmethod
    def from_scalars(cls, scalars) -> "Array":
        s = _buf(scalars, np.uint8, 32)
        return cls._new(lib().ft_array_from_scalars, _ptr(s), s.shape[0])

    @classmethod
    def from_small_scalars(cls, small) -> "Array":
        s = _buf(small, np.uint64)
        return cls._new(lib().ft_array_from_small_scalars, _ptr(s), s.shape[0])

    @classmethod
    def from_bytes_folded(cls, mem):
        m = _buf(mem, np.uint8)
        bad = ctypes.c_int64(-2)
        h = ctypes.c_void_p()
        check(lib().ft_array_from_bytes_folded(ctypes.byref(bad), ctypes.byref(h), _ptr(m), m.size))
        return Array(h), int(bad.value)

    @classmethod
    def from_bytes_affine(cls, mem) -> "Array":
        m = _buf(mem, np.uint8)
        return cls._new(lib().ft_array_from_bytes_affine, _ptr(m), m.size)

    @classmethod
    def from_bytes(cls, mem) -> "Array":
        m = _buf(mem, np.uint8)
        return cls._new(lib().ft_array_from_bytes, _ptr(m), m.size)

    @classmethod
    def from_packed(cls, mem) -> "Array":
        m = _buf(mem, np.uint8)
        return cls._new(lib().ftx_array_from_packed, _ptr(m), m.size)

    # ------------------------------------------------------------ export
    def _export(self, fn, width):
        n = len(self)
        out = np.zeros((n, width), dtype=np.uint8)
        check(fn(_ptr(out), out.size, self._h))
        return out

    def to_bytes_folded(self) -> np.ndarray:
        return self._export(lib().ft_array_to_bytes_folded, FOLDED)

    def to_bytes_affine(self) -> np.ndarray:
        return self._export(lib().ft_array_to_bytes_affine, AFFINE)

    def to_bytes(self) -> np.ndarray:
        return self._export(lib().ft_array_to_bytes, EXTENDED)

    def to_packed(self) -> np.ndarray:
        return self._export(lib().ftx_array_to_packed, PACKED)

    def device_view(self):
        p, s = ctypes.c_void_p(), ctypes.c_size_t()
        check(lib().ftx_array_device_view(self._h, ctypes.byref(p), ctypes.byref(s)))
        return p.value or 0, s.value

    # --------------------------------------------------- gather / scatter
    def get_subset(self, idxs) -> "Array":
        ix = _sz(idxs)
        return Array._new(lib().ft_array_get_subset, _ptr(ix), ix.size, self._h)

    def get_range(self, start, stop, step) -> "Array":
        return Array._new(lib().ft_array_get_range, start, stop, step, self._h)

    def assign_to_subset(self, idxs, src: "Array") -> None:
        ix = _sz(idxs)
        check(lib().ft_array_assign_to_subset(self._h, _ptr(ix), ix.size, src._h))

    def assign_zero_to_subset(self, idxs) -> None:
        ix = _sz(idxs)
        check(lib().ft_array_assign_zero_to_subset(self._h, _ptr(ix), ix.size))

    def assign_to_range(self, start, stop, step, src: "Array") -> None:
        check(lib().ft_array_assign_to_range(self._h, start, stop, step, src._h))

    def delete_subset(self, idxs) -> None:
        ix = _sz(idxs)
        check(lib().ft_array_delete_subset(self._h, _ptr(ix), ix.size))

    def delete_range(self, start, stop, step) -> None:
        check(lib().ft_array_delete_range(self._h, start, stop, step))

    def set_length(self, n: int) -> None:
        check(lib().ft_array_set_length(self._h, n))

    def mux(self, cond, iffalse: "Array") -> None:
        c = _buf(cond, np.int64)
        check(lib().ft_array_mux(self._h, _ptr(c), iffalse._h))

    def contains(self, other: "Array") -> np.ndarray:
        res = np.zeros(len(self), dtype=np.int64)
        check(lib().ft_array_contains(_ptr(res), self._h, other._h))
        return res

    # -------------------------------------------------------- arithmetic
    def add(self, summand: "Array") -> None:
        check(lib().ft_add(self._h, summand._h))

    def sub(self, subtrahend: "Array") -> None:
        check(lib().ft_sub(self._h, subtrahend._h))

    def neg(self) -> None:
        lib().ft_neg(self._h)
        check(lib().ftx_last_error())

    def scale(self, scalar) -> None:
        s = _buf(scalar, np.uint8).reshape(32)
        lib().ft_scale(self._h, _ptr(s))
        check(lib().ftx_last_error())

    def mul(self, scalars) -> None:
        s = _buf(scalars, np.uint8, 32)
        check(lib().ft_mul(self._h, _ptr(s), s.shape[0]))

    def scale_small(self, k: int, bits: int = 32) -> None:
        """self[i] = k * self[i] for k < 2^bits (a public bound)."""
        check(lib().ftx_scale_bounded(self._h, int(k), int(bits)))

    def mul_device(self, d_scalars_ptr: int, n: int) -> None:
        check(lib().ftx_mul_device(self._h, ctypes.c_void_p(d_scalars_ptr), n))

    def reduce_isum(self, idxs, summand: "Array") -> None:
        ix = _sz(idxs)
        check(lib().ft_reduce_isum(self._h, _ptr(ix), ix.size, summand._h))

    def index(self) -> np.ndarray:
        res = np.zeros(len(self), dtype=np.int64)
        lib().ft_index(_ptr(res), self._h)
        check(lib().ftx_last_error())
        return res

    def equal(self, other: "Array") -> np.ndarray:
        res = np.zeros(len(self), dtype=np.int64)
        check(lib().ft_equal(_ptr(res), self._h, other._h))
        return res

    def not_equal(self, other: "Array") -> np.ndarray:
        res = np.zeros(len(self), dtype=np.int64)
        check(lib().ft_not_equal(_ptr(res), self._h, other._h))
        return res

    def validate(self) -> int:
        r = ctypes.c_int64(-2)
        check(lib().ft_array_validate(ctypes.byref(r), self._h))
        return int(r.value)

    def prescan(self) -> None:
        check(lib().ft_array_prescan(self._h))

    def scan(self) -> None:
        check(lib().ft_array_scan(self._h))

    def reduce(self) -> None:
        check(lib().ft_array_reduce(self._h))

    def reduce_into(self, out: "Array", idx: int = 0) -> None:
        check(lib().ftx_reduce_into(out._h, idx, self._h))


def encrypt(pk32, m, r, plaintext_bits: int = 64):
    """ElGamal encryption under pk: returns (c1, c2)."""
    pk = _buf(pk32, np.uint8).reshape(32)
    mm = _buf(m, np.uint64)
    rr = _buf(r, np.uint8, 32)
    h1, h2 = ctypes.c_void_p(), ctypes.c_void_p()
    check(lib().ftx_encrypt(ctypes.byref(h1), ctypes.byref(h2), _ptr(pk), _ptr(mm), _ptr(rr), mm.size,
                            plaintext_bits))
    return Array(h1), Array(h2)


def encrypt_device(c1: Array, c2: Array, pk32, d_m: int, d_r: int, n: int, plaintext_bits: int = 64) -> None:
    pk = _buf(pk32, np.uint8).reshape(32)
    check(lib().ftx_encrypt_device(c1.handle, c2.handle, _ptr(pk), ctypes.c_void_p(d_m), ctypes.c_void_p(d_r), n,
                                   plaintext_bits))


def ct_add(c1: Array, c2: Array, d1: Array, d2: Array) -> None:
    """(c1, c2) += (d1, d2) in one launch."""
    check(lib().ftx_ct_add(c1.handle, c2.handle, d1.handle, d2.handle))


def ct_scan(c1: Array, c2: Array, exclusive: bool = False) -> None:
    """Prefix scan of both halves of a ciphertext array in one call."""
    check(lib().ftx_ct_scan(c1.handle, c2.handle, 1 if exclusive else 0))


def ct_sub(c1: Array, c2: Array, d1: Array, d2: Array) -> None:
    check(lib().ftx_ct_sub(c1.handle, c2.handle, d1.handle, d2.handle))


def rerandomise(c1: Array, c2: Array, pk32, r) -> None:
    """(c1, c2) += Enc(0; r) under pk, in place."""
    pk = _buf(pk32, np.uint8).reshape(32)
    rr = _buf(r, np.uint8, 32)
    check(lib().ftx_rerandomise(c1.handle, c2.handle, _ptr(pk), _ptr(rr), rr.shape[0]))


def rerandomise_device(c1: Array, c2: Array, pk32, d_r: int, n: int) -> None:
    pk = _buf(pk32, np.uint8).reshape(32)
    check(lib().ftx_rerandomise_device(c1.handle, c2.handle, _ptr(pk), ctypes.c_void_p(d_r), n))


DECRYPT_MAX_M = 1 << 24
NO_PLAINTEXT = np.uint64(0xFFFFFFFFFFFFFFFF)


def decrypt(c1: Array, c2: Array, sk32, m_max: int) -> np.ndarray:
    """Plaintexts j < m_max with c2 - sk*c1 = j*B; NO_PLAINTEXT where none."""
    sk = _buf(sk32, np.uint8).reshape(32)
    out = np.empty(len(c1), dtype=np.uint64)
    check(lib().ftx_decrypt(c1.handle, c2.handle, _ptr(sk), int(m_max), _ptr(out)))
    return out


def segmented_sum_csr(offsets, src: Array) -> Array:
    off = _buf(offsets, np.int32)
    return Array._new(lib().ftx_segmented_sum_csr, _ptr(off), off.size - 1, src.handle)


def segmented_sum_csr_device(out: Array, d_offsets: int, nseg: int, src: Array) -> None:
    check(lib().ftx_segmented_sum_csr_device(out.handle, ctypes.c_void_p(d_offsets), nseg, src.handle))


def ct_segmented_sum_csr_device(out1: Array, out2: Array, d_offsets: int, nseg: int, c1: Array, c2: Array) -> None:
    """ftx_ct_segmented_sum_csr_device: both halves of a ciphertext array over
    the same device offsets in the same launches."""
    check(lib().ftx_ct_segmented_sum_csr_device(out1.handle, out2.handle, ctypes.c_void_p(d_offsets), nseg,
                                                c1.handle, c2.handle))


class Batch:
    """ftx_batch: many independent array operations in one persistent launch
    replayed from a CUDA graph.  Keeps references to its arrays."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().ftx_batch_create(ctypes.byref(h)))
        self._h = h
        self._keep = []

    def add(self, res: Array, summand: Array) -> None:
        check(lib().ftx_batch_add(self._h, res.handle, summand.handle))
        self._keep += [res, summand]

    def scale_small(self, arr: Array, k: int, bits: int = 32) -> None:
        check(lib().ftx_batch_scale_bounded(self._h, arr.handle, int(k), int(bits)))
        self._keep.append(arr)

    def segmented_sum(self, out: Array, offsets, src: Array) -> None:
        off = _buf(offsets, np.int32)
        check(lib().ftx_batch_segmented_sum(self._h, out.handle, _ptr(off), off.size - 1, src.handle))
        self._keep += [out, src]

    def run(self) -> None:
        check(lib().ftx_batch_run(self._h))

    def info(self):
        a, b = ctypes.c_size_t(), ctypes.c_size_t()
        check(lib().ftx_batch_info(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def free(self) -> None:
        if self._h:
            lib().ftx_batch_free(self._h)
            self._h = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.ftx_batch_free(self._h)
            self._h = None


def tune(knob: int, value: int) -> None:
    check(lib().ftx_tune(knob, value))


def tune_get(knob: int) -> int:
    return int(lib().ftx_tune_get(knob))


TUNE_LADDER_BLOCK = 1
TUNE_SCALE_WINDOW = 3
TUNE_BATCH_ADD_PTS = 2


REQ_ENCRYPT, REQ_RERAND, REQ_SMUL, REQ_SEGSUM = 1, 2, 3, 4


class ServerArray(Array):
    """An output array a Server holds against its budget: free() (or garbage
    collection) hands it back through ftx_server_release while the server
    lives, and frees it as a plain array after the server is closed."""

    __slots__ = ("_srv",)

    def __init__(self, handle: ctypes.c_void_p, server: "Server"):
        super().__init__(handle)
        self._srv = server

    def free(self) -> None:
        if self._h:
            srv, self._srv = self._srv, None
            h, self._h = self._h, None
            if srv is not None and srv._h:
                check(lib().ftx_server_release(srv._h, h))
            else:
                lib().ft_array_free(h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            srv = getattr(self, "_srv", None)
            if srv is not None and srv._h:
                _lib._lib.ftx_server_release(srv._h, self._h)
            else:
                _lib._lib.ft_array_free(self._h)
            self._h = None


class Server:
    """ftx_server: continuous-batching request loop (see ftcrypto_gb300.h).
    Host buffers of a request are kept alive until its result is taken.
    Arrays a request creates are ServerArray objects charged to the budget
    until freed (release())."""

    def __init__(self, pk32, hbm_budget_bytes: int, slots: int = 8):
        pk = _buf(pk32, np.uint8).reshape(32)
        h = ctypes.c_void_p()
        check(lib().ftx_server_create(ctypes.byref(h), _ptr(pk), int(hbm_budget_bytes), int(slots)))
        self._h = h
        self._live = {}

    def _submit(self, req, keep, in_place):
        t = ctypes.c_uint64()
        check(lib().ftx_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        self._live[t.value] = (keep, in_place)
        return t.value

    def submit_encrypt(self, m, r, plaintext_bits: int = 64) -> int:
        mm, rr = _buf(m, np.uint64), _buf(r, np.uint8, 32)
        req = _lib.Request(op=REQ_ENCRYPT, n=mm.size, m=mm.ctypes.data, plaintext_bits=plaintext_bits,
                           r=rr.ctypes.data)
        return self._submit(req, (mm, rr), None)

    def submit_rerand(self, c1: Array, c2: Array, r) -> int:
        rr = _buf(r, np.uint8, 32)
        req = _lib.Request(op=REQ_RERAND, n=len(c1), r=rr.ctypes.data, c1=c1.handle.value, c2=c2.handle.value)
        return self._submit(req, (rr,), (c1, c2))

    def submit_smul(self, c1: Array, c2: Array, k) -> int:
        kk = _buf(k, np.uint8, 32)
        req = _lib.Request(op=REQ_SMUL, n=len(c1), k=kk.ctypes.data, c1=c1.handle.value, c2=c2.handle.value)
        return self._submit(req, (kk,), (c1, c2))

    def submit_segsum(self, c1: Array, c2: Array, offsets) -> int:
        off = _buf(offsets, np.int32)
        req = _lib.Request(op=REQ_SEGSUM, n=len(c1), offsets=off.ctypes.data, nseg=off.size - 1,
                           c1=c1.handle.value, c2=c2.handle.value)
        return self._submit(req, (off, c1, c2), None)

    def wait(self, ticket: int):
        """(c1, c2, queue_ms, latency_ms); new arrays for ENCRYPT / SEGSUM."""
        res = _lib.Result()
        check(lib().ftx_server_wait(self._h, ticket, ctypes.byref(res)))
        keep, in_place = self._live.pop(ticket)
        check(res.err)
        if in_place is not None:
            c1, c2 = in_place
        else:
            c1, c2 = ServerArray(ctypes.c_void_p(res.c1), self), ServerArray(ctypes.c_void_p(res.c2), self)
        return c1, c2, res.queue_ms, res.latency_ms

    def release(self, *arrays: ServerArray) -> None:
        """Hand outputs back: frees them and returns their bytes to the budget."""
        for a in arrays:
            a.free()

    def stats(self):
        a, b, c = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        check(lib().ftx_server_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def close(self) -> None:
        if self._h:
            lib().ftx_server_free(self._h)
            self._h = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib._lib is not None:
            _lib._lib.ftx_server_free(self._h)
            self._h = None
