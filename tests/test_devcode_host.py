"""The library's per-thread device arithmetic (csrc/fe.cuh, ge.cuh, smul.cuh),
compiled for the host over C stand-ins of its PTX carry primitives
(tests/host/ptx_emul.h), against Python integers and the oracle.  Catches
arithmetic errors without a GPU; the GPU tests check the real kernels."""
import ctypes
import os
import random
import subprocess

import numpy as np
import pytest

from libftcrypto_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
P = 2**255 - 19


@pytest.fixture(scope="module")
def hc(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("hc") / "devcode_host.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared",
                           '-DFT_HOST_EMULATION="../../tests/host/ptx_emul.h"', "-o", so,
                           os.path.join(HERE, "host", "devcode_host.cpp")])
    return ctypes.CDLL(so)


def w(x):
    return (ctypes.c_uint32 * 8)(*[(x >> (32 * i)) & 0xFFFFFFFF for i in range(8)])


def v(a):
    return sum(int(a[i]) << (32 * i) for i in range(8))


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_field_ops(hc):
    rnd = random.Random(5)
    edge = [0, 1, 2, 19, 38, P - 1, P, P + 1, 2 * P - 1, 2 * P, 2**255 - 1, 2**255, 2**256 - 1,
            2**256 - 38, 2**256 - 39, 2**256 - 20]
    vals = edge + [rnd.getrandbits(256) for _ in range(1500)]
    out = (ctypes.c_uint32 * 8)()
    for i, a in enumerate(vals):
        b = vals[(7 * i + 3) % len(vals)]
        for fn, want in ((hc.hc_fe_mul, a * b), (hc.hc_fe_add, a + b), (hc.hc_fe_sub, a - b)):
            fn(out, w(a), w(b))
            assert v(out) < 2**256 and v(out) % P == want % P
        hc.hc_fe_sq(out, w(a))
        assert v(out) < 2**256 and v(out) % P == a * a % P
        hc.hc_fe_canon(out, w(a))
        assert v(out) == a % P
    for a in vals[:100]:
        hc.hc_fe_invert(out, w(a))
        assert v(out) % P == pow(a, P - 2, P)


def test_wide_products_exact(hc):
    """mul_wide / sqr_wide return the exact 512-bit product (so the fold, and
    every coordinate after it, is the same whatever the accumulation order):
    random operands, limbs of all ones, single set limbs."""
    rnd = random.Random(9)
    M = 2**256 - 1
    vals = [0, 1, M, M - 1, 2**255, 2**224, 2**32 - 1, (2**32 - 1) << 224]
    vals += [sum(((2**32 - 1) if (m >> k) & 1 else 0) << (32 * k) for k in range(8)) for m in range(0, 256, 7)]
    vals += [rnd.getrandbits(256) for _ in range(3000)]
    t = (ctypes.c_uint32 * 16)()

    def v16(x):
        return sum(int(x[i]) << (32 * i) for i in range(16))
    for i, a in enumerate(vals):
        b = vals[(11 * i + 5) % len(vals)]
        hc.hc_mul_wide(t, w(a), w(b))
        assert v16(t) == a * b
        hc.hc_sqr_wide(t, w(a))
        assert v16(t) == a * a


def test_mul_sq_words(hc):
    """fe_mul / fe_sq return exactly fold(product): v = lo + 38 hi twice,
    then a last + 38 for the carry (the words every coordinate depends on)."""
    M = 2**256 - 1

    def fold(t):
        v = (t & M) + 38 * (t >> 256)
        v = (v & M) + 38 * (v >> 256)
        return (v & M) + 38 * (v >> 256)
    rnd = random.Random(10)
    vals = [0, 1, M, M - 1, 2**255 - 19, 2**255, M - 37, M - 38] + [rnd.getrandbits(256) for _ in range(3000)]
    vals += [M - rnd.getrandbits(40) for _ in range(200)]
    out = (ctypes.c_uint32 * 8)()
    for i, a in enumerate(vals):
        b = vals[(13 * i + 1) % len(vals)]
        hc.hc_fe_mul(out, w(a), w(b))
        assert v(out) == fold(a * b)
        hc.hc_fe_sq(out, w(a))
        assert v(out) == fold(a * a)


def test_group_and_smul(hc, orc):
    g = synth.rng(3)
    n = 48
    sc = synth.scalars_mod_L(g, n)
    for i, x in enumerate([0, 1, synth.L - 1, 2**256 - 1, 2**255 + 12345]):
        sc[i] = synth.int_to_scalar(x)
    p1 = orc.from_scalars(sc)
    p2 = orc.from_scalars(np.ascontiguousarray(sc[::-1]))
    a = p1.copy()
    hc.hc_add(ptr(a), ptr(p2), n)
    assert (orc.encode(a) == orc.encode(orc.add(p1, p2))).all()
    s = p1.copy()
    hc.hc_sub(ptr(s), ptr(p2), n)
    assert (orc.encode(s) == orc.encode(orc.sub(p1, p2))).all()
    m = p1.copy()
    hc.hc_mul(ptr(m), ptr(sc), n)
    om = orc.mul(p1, sc)
    assert (m == om).all()  # same formula sequence: identical coordinates
    c = np.zeros_like(p1)
    base = orc.from_scalars(synth.int_to_scalar(1)[None])
    hc.hc_enc_comb(ptr(c), ptr(sc), n, 52, ptr(base))  # the radix-32 comb, 52 rows
    assert (orc.encode(c) == orc.encode(p1)).all()
    e = np.zeros((n, 32), np.uint8)
    hc.hc_encode(ptr(e), ptr(om), n)
    assert (e == orc.encode(om)).all()


@pytest.mark.parametrize("nt", [384, 448])
def test_hybrid_table_ladder(hc, orc, nt):
    """The ladder over the tensor-memory kernel's tables (half in shared
    memory, half in an emulated TMEM that aborts on an out-of-range column)
    gives the oracle's coordinates for threads in every warp slot."""
    g = synth.rng(nt)
    n = nt + 40  # every thread of a block, then a second block's first warps
    sc = synth.scalars_mod_L(g, n)
    for i, x in enumerate([0, 1, synth.L - 1, 2**256 - 1, 2**255 + 12345]):
        sc[i] = synth.int_to_scalar(x)
    p = orc.from_scalars(np.ascontiguousarray(sc[::-1]), threads=8)
    m = p.copy()
    assert hc.hc_mul_hybrid(ptr(m), ptr(sc), n, nt) == 0
    assert (m == orc.mul(p, sc, threads=8)).all()


@pytest.mark.parametrize("w", [2, 3, 4])
def test_bounded_small_scalar_ladder(hc, orc, w):
    """The small-scalar ladder of window width w in the window count of
    windows.h is exact for every k < 2^bits, including the largest k of each
    bound (where a window fewer would lose the recoding's carry)."""
    g = synth.rng(12 + w)
    for bits in list(range(1, 17)) + [20, 23, 24, 27, 28, 31, 32]:
        ks = {0, 1, (1 << bits) - 1, (1 << bits) - 2, (1 << bits) // 2}
        ks |= {int(x) for x in g.integers(0, 1 << bits, 3, dtype=np.uint64)}
        ks = np.array(sorted(ks), dtype=np.uint32)
        p = orc.from_scalars(synth.scalars_mod_L(g, ks.size))
        m = p.copy()
        assert hc.hc_mul_u32_bits(ptr(m), ptr(ks), ks.size, bits, w) == 0
        want = np.stack([orc.scale(p[i:i + 1], synth.int_to_scalar(int(k)))[0] for i, k in enumerate(ks)])
        assert (orc.encode(m) == orc.encode(want)).all(), (w, bits)


def test_decode_and_small_comb(hc, orc):
    g = synth.rng(4)
    good = orc.encode(orc.from_scalars(synth.scalars_mod_L(g, 20)))
    inp = np.concatenate([good, g.integers(0, 256, (100, 32), dtype=np.uint8)])
    d = np.zeros((inp.shape[0], 128), np.uint8)
    hc.hc_decode.restype = ctypes.c_longlong
    bad = hc.hc_decode(ptr(d), ptr(inp), inp.shape[0])
    od, obad = orc.decode(inp)
    assert bad == obad
    assert (orc.encode(d) == orc.encode(od)).all()
    m = np.array([0, 1, 255, 2**32, 2**64 - 1] + list(range(7, 22)), dtype=np.uint64)
    small = orc.small_to_scalars(m)
    c = np.zeros((len(m), 128), np.uint8)
    base = orc.from_scalars(synth.int_to_scalar(1)[None])
    rows = hc.hc_enc_digits(64)
    assert rows == 14
    hc.hc_enc_comb(ptr(c), ptr(small), len(m), rows, ptr(base))  # uint64 values: 14 rows
    assert (orc.encode(c) == orc.encode(orc.from_scalars(small))).all()
    # a full-width scalar and the largest 256-bit one need all 52 rows
    big = np.stack([synth.int_to_scalar(2**256 - 1), synth.int_to_scalar(2**255 + 12345)])
    cb = np.zeros((2, 128), np.uint8)
    hc.hc_enc_comb(ptr(cb), ptr(big), 2, 52, ptr(base))
    assert (orc.encode(cb) == orc.encode(orc.from_scalars(big))).all()


def test_short_ladder_matches_full(hc, orc):
    g = synth.rng(6)
    n = 40
    p = orc.from_scalars(synth.scalars_mod_L(g, n))
    k = g.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    k[:4] = [0, 1, 2**32 - 1, 1000]
    m = p.copy()
    hc.hc_mul_u32(ptr(m), ptr(k), n)
    full = orc.mul(p, orc.small_to_scalars(k.astype(np.uint64)))
    assert (orc.encode(m) == orc.encode(full)).all()
