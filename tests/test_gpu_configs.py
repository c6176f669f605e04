"""Every benchmark configuration at its full size, byte for byte against the
oracle: the canonical 32-byte encoding of every output point of the CUDA
path (through the C ABI) equals the oracle's encoding of the same operation
on the same inputs.

  ciphertext add   two arrays of 65,536 ElGamal ciphertexts, m in {0,1}:
                   all 65,536 sums (ftx_ct_add and two ft_add calls), plus
                   decryption to m1 + m2 (ft_add, ftcrypto.cu:1089-1110)
  encrypt + mult   1,048,576 ciphertexts of 8-bit plaintexts, then both
                   halves times a per-element secret scalar mod L: all
                   2,097,152 output points (ft_mul, ftcrypto.cu:986-1011;
                   the oracle encrypts in the reference's composition).
                   Host inputs, as in the end-to-end step: the encryption
                   and each ladder run in two launches and the exports
                   copy the first part while the second computes
  reductions       the sum of 16,777,216 ciphertexts (ft_array_reduce,
                   ftcrypto.cu:1414-1471), the segmented sum of the same
                   points into 1,048,576 CSR segments (ftcrypto.cu:1113-1217),
                   every one of the 2 x 4,194,304 inclusive scan outputs and
                   the exclusive scan of one half (ftcrypto.cu:1474-1586)
  uneven batch     all 4,096 arrays of the mixed add / scale / segmented-sum
                   workload, batched (one persistent launch from a CUDA graph)
                   and one call per array

The reduction inputs are ciphertexts encrypted on the GPU and exported in
the packed layout (the encryption itself is checked by the encrypt + mult
case); the oracle sums them on all host cores and encodes with batched
inversion (both checked against the serial oracle on the CPU).
"""
import os

import numpy as np
import pytest

from libftcrypto_gb300 import synth

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def keypair(ft, orc, g):
    sk = synth.scalars_mod_L(g, 1)
    pk = orc.encode(orc.from_scalars(sk))[0]
    assert (ft.Array.from_scalars(sk).to_bytes_folded()[0] == pk).all()
    return sk[0], pk


def mismatches(got, want):
    assert got.shape == want.shape
    return int((got != want).any(axis=1).sum())


def test_ct_add_65536(ft, orc):
    g = synth.rng(1001)
    sk, pk = keypair(ft, orc, g)
    n = 65536
    ma, mb = synth.plaintexts(g, n, 1), synth.plaintexts(g, n, 1)
    ra, rb = synth.scalars_mod_L(g, n), synth.scalars_mod_L(g, n)
    a1, a2 = ft.encrypt(pk, ma, ra, 1)
    b1, b2 = ft.encrypt(pk, mb, rb, 1)
    p1, p2 = a1.get_range(0, n, 1), a2.get_range(0, n, 1)
    ft.ct_add(a1, a2, b1, b2)        # both halves in one launch
    p1.add(b1)                       # the drop-in: two ft_add calls
    p2.add(b2)

    o1, o2 = orc.encrypt(pk, ma, ra, threads=THREADS)
    q1, q2 = orc.encrypt(pk, mb, rb, threads=THREADS)
    want1 = orc.encode(orc.add(o1, q1, threads=THREADS), threads=THREADS)
    want2 = orc.encode(orc.add(o2, q2, threads=THREADS), threads=THREADS)
    for c1, c2 in ((a1, a2), (p1, p2)):
        assert mismatches(c1.to_bytes_folded(), want1) == 0
        assert mismatches(c2.to_bytes_folded(), want2) == 0
    assert (ft.decrypt(a1, a2, sk, 4) == ma + mb).all()


def test_encrypt_mul_1M(ft, orc):
    g = synth.rng(1002)
    _, pk = keypair(ft, orc, g)
    n = 1 << 20
    m = synth.plaintexts(g, n, 255)
    r = synth.scalars_mod_L(g, n)
    k = synth.scalars_mod_L(g, n)
    c1, c2 = ft.encrypt(pk, m, r, 8)
    c1.mul(k)
    c2.mul(k)
    got1, got2 = c1.to_bytes_folded(), c2.to_bytes_folded()
    del c1, c2
    o1, o2 = orc.encrypt(pk, m, r, threads=THREADS)
    want1 = orc.encode(orc.mul(o1, k, threads=THREADS), threads=THREADS)
    del o1
    want2 = orc.encode(orc.mul(o2, k, threads=THREADS), threads=THREADS)
    assert mismatches(got1, want1) == 0
    assert mismatches(got2, want2) == 0


@pytest.fixture(scope="module")
def ct16m(ft, orc):
    """16,777,216 ciphertexts of m in {0,1}, encrypted on the GPU."""
    g = synth.rng(1003)
    _, pk = keypair(ft, orc, g)
    n = 1 << 24
    m = synth.plaintexts(g, n, 1)
    r = synth.scalars_mod_L(g, n)
    c1, c2 = ft.encrypt(pk, m, r, 1)
    del r
    off = synth.csr_offsets(g, n, 1 << 20)
    yield c1, c2, off
    c1.free()
    c2.free()


def test_reduce_and_segsum_16M(ft, orc, ct16m):
    c1, c2, off = ct16m
    n = len(c1)
    for half in (c1, c2):
        s = half.get_range(0, n, 1)
        s.reduce()                                    # ft_array_reduce: shrinks to 1
        assert len(s) == 1
        got_sum = s.to_bytes_folded()
        got_seg = ft.segmented_sum_csr(off, half).to_bytes_folded()
        pts = half.to_packed()
        want_sum = orc.encode(orc.reduce(pts, threads=THREADS))
        want_seg = orc.encode(orc.segsum_csr(off, pts, threads=THREADS), threads=THREADS)
        del pts
        assert mismatches(got_sum, want_sum) == 0
        assert mismatches(got_seg, want_seg) == 0


def test_reduce_isum_16M_keys(ft, orc, ct16m):
    """ft_reduce_isum over the same 16,777,216 points with the segment of
    every point as its key (shuffled), accumulated into res = the segment
    sums themselves: res ends as twice the segmented sum."""
    c1, _, off = ct16m
    g = synth.rng(1004)
    nseg = len(off) - 1
    keys = synth.segment_ids(off)
    perm = g.permutation(len(keys))
    src = c1.get_subset(perm)
    res = ft.segmented_sum_csr(off, c1)
    res.reduce_isum(keys[perm], src)
    del src
    got = res.to_bytes_folded()
    seg = orc.segsum_csr(off, c1.to_packed(), threads=THREADS)
    want = orc.encode(orc.add(seg, seg, threads=THREADS), threads=THREADS)
    assert got.shape == (nseg, 32)
    assert mismatches(got, want) == 0


def test_scan_4M(ft, orc):
    g = synth.rng(1005)
    _, pk = keypair(ft, orc, g)
    n = 1 << 22
    m = synth.plaintexts(g, n, 1)
    r = synth.scalars_mod_L(g, n)
    c1, c2 = ft.encrypt(pk, m, r, 1)
    for half, exclusive in ((c1, False), (c2, False), (c1, True)):
        pts = half.to_packed()
        s = half.get_range(0, n, 1)
        if exclusive:
            s.prescan()
        else:
            s.scan()
        got = s.to_bytes_folded()
        del s
        want = orc.encode(orc.scan(pts, exclusive, threads=THREADS), threads=THREADS)
        del pts
        assert mismatches(got, want) == 0


def test_uneven_batch_all_4096_arrays(ft, orc):
    """All 4,096 arrays of the uneven mix (24.8 M ciphertexts), each array a
    range of a pool of 131,072 points: batched and one call per array, every
    output against the oracle (scale by k <= 1000 on the oracle side by
    double-and-add, the ladder's group element)."""
    g = synth.rng(1006)
    work = synth.uneven_mix(g, n_arrays=4096)
    P = 1 << 17
    sc = synth.scalars_mod_L(g, P)
    pool = ft.Array.from_scalars(sc)
    opool = orc.from_scalars(sc, threads=THREADS)
    assert mismatches(pool.to_bytes_folded(), orc.encode(opool, threads=THREADS)) == 0
    offs = [int(g.integers(0, P - w["len"] + 1)) for w in work]

    def make():
        arrs = []
        for w, o in zip(work, offs):
            n = w["len"]
            c1, c2 = pool.get_range(o, o + n, 1), pool.get_range(P - n - o, P - o, 1)
            ex = {}
            if w["op"] == "add":
                ex["s1"], ex["s2"] = pool.get_range(0, n, 1), pool.get_range(P - n, P, 1)
            elif w["op"] == "segsum":
                nseg = len(w["offsets"]) - 1
                ex["o1"], ex["o2"] = ft.Array.init_scalar(nseg), ft.Array.init_scalar(nseg)
            arrs.append((c1, c2, ex))
        return arrs

    batched, plain = make(), make()
    b = ft.Batch()
    for w, (c1, c2, ex) in zip(work, batched):
        if w["op"] == "add":
            b.add(c1, ex["s1"])
            b.add(c2, ex["s2"])
        elif w["op"] == "scale":
            b.scale_small(c1, w["k"], w["bits"])
            b.scale_small(c2, w["k"], w["bits"])
        else:
            b.segmented_sum(ex["o1"], w["offsets"], c1)
            b.segmented_sum(ex["o2"], w["offsets"], c2)
    b.run()
    for w, (c1, c2, ex) in zip(work, plain):
        if w["op"] == "add":
            c1.add(ex["s1"])
            c2.add(ex["s2"])
        elif w["op"] == "scale":
            c1.scale_small(w["k"], w["bits"])
            c2.scale_small(w["k"], w["bits"])
        else:
            nseg = len(ex["o1"])
            ex["o1"].free()
            ex["o2"].free()
            ex["o1"], ex["o2"] = ft.segmented_sum_csr(w["offsets"], c1), ft.segmented_sum_csr(w["offsets"], c2)
            assert len(ex["o1"]) == nseg

    bad, compared = 0, 0
    for w, o, bt, pl in zip(work, offs, batched, plain):
        n = w["len"]
        x1, x2 = opool[o:o + n], opool[P - n - o:P - o]
        if w["op"] == "add":
            want = (orc.add(x1, opool[0:n]), orc.add(x2, opool[P - n:P]))
        elif w["op"] == "scale":
            want = (orc.scale_u64(x1, w["k"], threads=THREADS), orc.scale_u64(x2, w["k"], threads=THREADS))
        else:
            want = (orc.segsum_csr(w["offsets"], x1), orc.segsum_csr(w["offsets"], x2))
        want = [orc.encode(x, threads=THREADS) for x in want]
        for form in (bt, pl):
            c1, c2, ex = form
            outs = (ex["o1"], ex["o2"]) if w["op"] == "segsum" else (c1, c2)
            for arr, wv in zip(outs, want):
                bad += mismatches(arr.to_bytes_folded(), wv)
                compared += wv.shape[0]
    b.free()
    outputs = sum(len(w["offsets"]) - 1 if w["op"] == "segsum" else w["len"] for w in work)
    assert compared == 2 * 2 * outputs  # both forms, both halves of every array
    assert bad == 0
