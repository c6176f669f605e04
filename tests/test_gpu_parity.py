"""Parity of the CUDA library (through its C ABI) with the oracle and the
reference's golden vectors: every output compared as canonical folded
encodings, which must be byte-identical (bit-exact integer arithmetic; no
tolerance)."""
import numpy as np
import pytest

from conftest import hx, hxs
from libftcrypto_gb300 import synth

pytestmark = pytest.mark.gpu


def enc(a):
    return [bytes(e).hex() for e in a]


def rand_points(orc, g, n):
    return orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)


def upload(ft, pts):
    return ft.Array.from_packed(pts)


# ------------------------------------------------------------------ golden

def test_run_tests_cases(ft, golden):
    a = ft.Array.from_small_scalars(np.arange(9))
    a.reduce()
    assert len(a) == 1
    assert enc(a.to_bytes_folded()) == [golden["reduce_0_8"]]
    s = ft.Array.from_small_scalars(np.arange(7))
    s.scan()
    assert enc(s.to_bytes_folded()) == golden["scan_0_6"]
    ex = golden["isum_example"]
    r = ft.Array.from_small_scalars(ex["res"])
    r.reduce_isum(ex["keys"], ft.Array.from_small_scalars(ex["src"]))
    assert enc(r.to_bytes_folded()) == ex["out"]
    five = ft.Array.from_small_scalars([5])
    five2 = ft.Array.from_small_scalars([5])
    eq1 = int(five.equal(five2)[0])
    five2.add(five)
    assert [eq1, int(five.equal(five2)[0])] == golden["equal_example"]
    arr = ft.Array.from_small_scalars(range(1, 8))
    probe = ft.Array.from_small_scalars([3, 5, 8, 2])
    assert list(probe.contains(arr)) == golden["contains_example"]
    z = ft.Array.init_scalar(16)
    assert enc(z.to_bytes_folded()) == [golden["identity"]] * 16
    # in-place ft_add(a, a) of run_tests.cc:82-88
    sub = z.get_subset([3, 7, 8])
    sub.add(sub)
    assert enc(sub.to_bytes_folded()) == [golden["identity"]] * 3
    # affine round trip validates (run_tests.cc:92-103)
    b = ft.Array.from_small_scalars(range(1, 17))
    a3 = ft.Array.from_bytes_affine(b.to_bytes_affine())
    assert a3.validate() == -1


def test_scalarmult_golden(ft, golden):
    cs = golden["smul"]
    pts, bad = ft.Array.from_bytes_folded(hxs(c["point"] for c in cs))
    assert bad == -1
    pts.mul(hxs(c["scalar"] for c in cs))
    assert enc(pts.to_bytes_folded()) == [c["out"] for c in cs]
    sb = golden["smul_base"]
    b = ft.Array.from_scalars(hxs(c["scalar"] for c in sb))
    assert enc(b.to_bytes_folded()) == [c["ladder"] for c in sb]


def test_add_sub_neg_golden(ft, golden):
    cs = golden["addsub"]
    a, _ = ft.Array.from_bytes_folded(hxs(c["a"] for c in cs))
    b, _ = ft.Array.from_bytes_folded(hxs(c["b"] for c in cs))
    s, _ = ft.Array.from_bytes_folded(hxs(c["a"] for c in cs))
    s.add(b)
    assert enc(s.to_bytes_folded()) == [c["sum"] for c in cs]
    d, _ = ft.Array.from_bytes_folded(hxs(c["a"] for c in cs))
    d.sub(b)
    assert enc(d.to_bytes_folded()) == [c["diff"] for c in cs]
    a.neg()
    assert enc(a.to_bytes_folded()) == [c["neg_a"] for c in cs]


def test_decode_golden(ft, golden):
    cs = golden["decode"]
    arr, bad = ft.Array.from_bytes_folded(hxs(c["in"] for c in cs))
    assert bad == max(i for i, c in enumerate(cs) if not c["ok"])
    assert enc(arr.to_bytes_folded()) == [c["reenc"] for c in cs]
    for i, c in enumerate(cs):
        one = arr.get_subset([i])
        assert (one.validate() == -1) == bool(c["valid"]), i


def test_contains_large_with_duplicates_and_empty(ft):
    """ft_array_contains by the device hash table of encodings: membership of
    k*B in {k'*B} is membership of k in {k'} (distinct k < L give distinct
    points); duplicates, the identity (k = 0) and empty arrays included."""
    g = synth.rng(16)
    k2 = g.integers(0, 5000, 3000).astype(np.uint64)
    k1 = g.integers(0, 8000, 5000).astype(np.uint64)
    a1, a2 = ft.Array.from_small_scalars(k1), ft.Array.from_small_scalars(k2)
    assert (a1.contains(a2) == np.isin(k1, k2).astype(np.int64)).all()
    empty = ft.Array.init_scalar(0)
    assert len(empty.contains(a2)) == 0
    assert (a1.contains(empty) == 0).all()


def ref_contains(orc, a1, a2):
    """The reference's ft_array_contains (ftcrypto.cu:1046-1070) on the
    oracle: res[j] = OR over i of ge25519_equal(a2[i], a1[j]), where equal
    is iszero(a2[i] - a1[j]) by the projective formulas (ftcrypto.cu:170-190)."""
    n1, n2 = a1.shape[0], a2.shape[0]
    eq = orc.equal(np.repeat(a2, n1, axis=0), np.tile(a1, (n2, 1))).reshape(n2, n1)
    return eq.any(axis=0).astype(np.int64)


def test_contains_on_and_off_the_curve(ft, orc, golden):
    """ft_array_contains is membership of canonical encodings.  On the curve
    that is the reference's answer.  Off the curve (the reference's results
    for rejected encodings) it is not: the reference's projective test
    iszero(p - q) needs the curve equation, so it reports an off-curve point
    as absent even from an array holding the same point, while this library
    reports it present (same encoding).  Both rules are pinned here."""
    dec = golden["decode"]
    pts, _ = orc.decode(hxs(c["in"] for c in dec))
    ok = np.array([bool(c["ok"]) for c in dec])
    g = synth.rng(17)
    on = orc.from_scalars(synth.scalars_mod_L(g, 40), threads=4)
    a1 = np.concatenate([pts, on])
    a2 = np.concatenate([pts[::3], on[::2]])
    got = ft.Array.from_packed(a1).contains(ft.Array.from_packed(a2))
    e1, e2 = orc.encode(a1), orc.encode(a2)
    by_encoding = (e1[:, None, :] == e2[None, :, :]).all(-1).any(axis=1).astype(np.int64)
    assert (got == by_encoding).all()
    ref = ref_contains(orc, a1, a2)
    on_curve = np.concatenate([ok, np.ones(len(on), dtype=bool)])
    assert (got[on_curve] == ref[on_curve]).all()
    # the divergence: off-curve points found by encoding, absent for the reference
    off = ~on_curve
    assert off.any() and (got[off] == by_encoding[off]).all()
    assert ((ref[off] == 0) | (got[off] == 1)).all()
    assert (got[off] != ref[off]).any()


def test_off_curve_points_follow_the_formulas(ft, orc, golden):
    """Decoded points include the reference's results for rejected encodings
    (not on the curve); multiplication and addition still run the same field
    operations as the oracle, word for word."""
    cs = golden["decode"]
    arr, bad = ft.Array.from_bytes_folded(hxs(c["in"] for c in cs))
    assert bad >= 0  # the fixture holds rejected encodings
    pts = arr.to_packed()
    k = synth.scalars_mod_L(synth.rng(15), len(cs))
    M = ft.Array.from_packed(pts)
    M.mul(k)
    assert (M.to_packed() == orc.mul(pts, k, threads=8)).all()
    rev = np.ascontiguousarray(pts[::-1])
    A = ft.Array.from_packed(pts)
    A.add(ft.Array.from_packed(rev))
    assert (A.to_packed() == orc.add(pts, rev)).all()


def test_affine_raw_golden(ft, golden):
    af = golden["affine"]
    a, _ = ft.Array.from_bytes_folded(hxs(c["enc"] for c in af))
    assert enc(a.to_bytes_affine()) == [c["affine"] for c in af]
    raw = golden["raw160"]
    r = ft.Array.from_bytes(hxs(c["raw"] for c in raw))
    assert enc(r.to_bytes_folded()) == [c["enc"] for c in raw]
    back = ft.Array.from_bytes(r.to_bytes())
    assert enc(back.to_bytes_folded()) == [c["enc"] for c in raw]
    q = golden["validate_neg_quirk"]
    assert (ft.Array.from_bytes(hx(q["raw"])).validate() == -1) == bool(q["valid"])


def test_encrypt_golden(ft, golden):
    e = golden["encrypt"]
    cs = e["cases"]
    c1, c2 = ft.encrypt(hx(e["pk"]), [c["m"] for c in cs], hxs(c["r"] for c in cs), 64)
    assert enc(c1.to_bytes_folded()) == [c["c1"] for c in cs]
    assert enc(c2.to_bytes_folded()) == [c["c2"] for c in cs]
    small = [i for i, c in enumerate(cs) if c["m"] < 256]
    d1, d2 = ft.encrypt(hx(e["pk"]), [cs[i]["m"] for i in small], hxs(cs[i]["r"] for i in small), 8)
    assert enc(d2.to_bytes_folded()) == [cs[i]["c2"] for i in small]
    with pytest.raises(ft.FtError) as ei:
        ft.encrypt(hx(e["pk"]), [256], hxs([cs[0]["r"]]), 8)
    assert ei.value.code == 3


# ------------------------------------------------------------ element-wise

@pytest.mark.parametrize("n", [0, 1, 2, 31, 255, 256, 257, 1000])
def test_add_sub_mul_vs_oracle(ft, orc, n):
    g = synth.rng(100 + n)
    a = rand_points(orc, g, n)
    b = rand_points(orc, g, n)
    k = synth.scalars_mod_L(g, n)
    A = upload(ft, a)
    A.add(upload(ft, b))
    assert (A.to_bytes_folded() == orc.encode(orc.add(a, b))).all()
    A.sub(upload(ft, b))
    assert (A.to_bytes_folded() == orc.encode(a)).all()
    M = upload(ft, a)
    M.mul(k)
    om = orc.mul(a, k, threads=8)
    assert (M.to_packed() == om).all()  # same formulas: identical coordinates
    assert (M.to_bytes_folded() == orc.encode(om)).all()


@pytest.mark.parametrize("block", [128, 192, 224, 384, 448])
def test_ladder_block_sizes(ft, orc, block):
    """Every ladder kernel (tables in shared memory, or half in tensor memory
    for 384 and 448) gives the oracle's coordinates word for word, with
    partial last blocks and edge scalars."""
    g = synth.rng(40 + block)
    before = ft.tune_get(ft.TUNE_LADDER_BLOCK)
    ft.tune(ft.TUNE_LADDER_BLOCK, block)
    try:
        for n in (1, block - 1, block + 1, 3 * block + 37):
            a = rand_points(orc, g, n)
            k = synth.scalars_mod_L(g, n)
            edge = [0, 1, synth.L - 1, 2**255 - 1, 2**256 - 1]
            for j, v in enumerate(edge[:n]):
                k[j] = synth.int_to_scalar(v)
            M = upload(ft, a)
            M.mul(k)
            assert (M.to_packed() == orc.mul(a, k, threads=8)).all(), n
    finally:
        ft.tune(ft.TUNE_LADDER_BLOCK, before)


def test_aliasing_and_size_mismatch(ft, orc):
    g = synth.rng(7)
    a = rand_points(orc, g, 33)
    A = upload(ft, a)
    A.add(A)
    assert (A.to_bytes_folded() == orc.encode(orc.add(a, a))).all()
    with pytest.raises(ft.FtError) as e:
        A.add(upload(ft, a[:5]))
    assert e.value.code == 2
    with pytest.raises(ft.FtError) as e:
        A.mul(synth.scalars_mod_L(g, 5))
    assert e.value.code == 2


def test_scale_and_edge_scalars(ft, orc):
    g = synth.rng(8)
    a = rand_points(orc, g, 70)
    for v in [0, 1, 2, synth.L - 1, synth.L, 2**255 - 1, 2**256 - 1, 2**252 + 77]:
        s = synth.int_to_scalar(v)
        A = upload(ft, a)
        A.scale(s)
        assert (A.to_bytes_folded() == orc.encode(orc.scale(a, s))).all(), v


def test_fixed_base_edge_scalars(ft, orc):
    """from_scalars and encryption at scalars the reference's recoding
    truncates (top digit above 8, from ~9 * 2^252) and around them: the
    radix-32 comb reproduces the reference's points."""
    g = synth.rng(12)
    vals = [0, 1, 2, synth.L - 1, synth.L, 2**252, 8 * 2**252 + 5, 9 * 2**252 - 1, 9 * 2**252,
            2**255 - 1, 2**255, 2**255 + 12345, 2**256 - 2**252, 2**256 - 1]
    s = np.stack([synth.int_to_scalar(v) for v in vals] + list(synth.scalars_mod_L(g, 50)))
    want = orc.encode(orc.from_scalars(s, threads=8))
    assert (ft.Array.from_scalars(s).to_bytes_folded() == want).all()
    sk = synth.scalars_mod_L(g, 1)
    pk = ft.Array.from_scalars(sk).to_bytes_folded()[0]
    m = g.integers(0, 256, size=len(s), dtype=np.uint64)
    c1, c2 = ft.encrypt(pk, m, s, 8)
    o1, o2 = orc.encrypt(pk, m, s, threads=8)
    assert (c1.to_bytes_folded() == orc.encode(o1)).all()
    assert (c2.to_bytes_folded() == orc.encode(o2)).all()


def test_export_into_pinned_memory(ft, orc):
    """Exports into pinned host memory, at an aligned and an unaligned
    address, equal the exports into pageable memory."""
    torch = pytest.importorskip("torch")
    import ctypes
    g = synth.rng(13)
    n = 1000
    a = ft.Array.from_scalars(synth.scalars_mod_L(g, n))
    L = ft.api.lib()
    for fn, width in ((L.ft_array_to_bytes, 160), (L.ft_array_to_bytes_folded, 32), (L.ft_array_to_bytes_affine, 64)):
        want = np.zeros(n * width, np.uint8)
        ft.check(fn(want.ctypes.data_as(ctypes.c_void_p), want.size, a.handle))
        for off in (0, 1):
            pin = torch.zeros(n * width + 16, dtype=torch.uint8).pin_memory()
            ptr = ctypes.c_void_p(pin.data_ptr() + off)
            ft.check(fn(ptr, n * width, a.handle))
            got = pin.numpy()[off:off + n * width]
            assert (got == want).all(), (width, off)
    assert (want.reshape(n, 64)[:, :32] != 0).any()


def test_large_exports_equal_concatenated_ranges(ft):
    """An export of 600,001 points equals the concatenated exports of three
    sub-ranges (taken by get_range), in every format; the raw import of the
    raw export gives the points back."""
    import ctypes
    g = synth.rng(14)
    n = 600_001
    a = ft.Array.from_small_scalars(g.integers(0, 1 << 40, n).astype(np.uint64))
    L = ft.api.lib()
    cuts = [0, 200_000, 400_000, n]
    parts = [a.get_range(lo, hi, 1) for lo, hi in zip(cuts, cuts[1:])]
    for fn, width in ((L.ft_array_to_bytes, 160), (L.ft_array_to_bytes_folded, 32), (L.ft_array_to_bytes_affine, 64),
                      (L.ftx_array_to_packed, 128)):
        got = np.zeros(n * width, np.uint8)
        ft.check(fn(got.ctypes.data_as(ctypes.c_void_p), got.size, a.handle))
        want = []
        for p in parts:
            w = np.zeros(len(p) * width, np.uint8)
            ft.check(fn(w.ctypes.data_as(ctypes.c_void_p), w.size, p.handle))
            want.append(w)
        assert (got == np.concatenate(want)).all(), width
        if width == 160:  # and the raw import of all of it gives the points back
            back = ft.Array.from_bytes(got.reshape(n, 160))
            assert (back.to_bytes_folded() == a.to_bytes_folded()).all()


def test_constructors(ft, orc):
    g = synth.rng(9)
    s = synth.scalars_mod_L(g, 300)
    s[0] = 0
    assert (ft.Array.from_scalars(s).to_bytes_folded() == orc.encode(orc.from_scalars(s, threads=8))).all()
    m = g.integers(0, 2**63, 200, dtype=np.uint64)
    m[:3] = [0, 1, np.uint64(2**64 - 1)]
    got = ft.Array.from_small_scalars(m).to_bytes_folded()
    assert (got == orc.encode(orc.from_scalars(orc.small_to_scalars(m), threads=8))).all()
    one = synth.int_to_scalar(123456789)
    A = ft.Array.init_scalar(77, one)
    assert (A.to_bytes_folded() == orc.encode(orc.from_scalars(np.tile(one, (77, 1))))).all()
    P = ft.Array.init_point(9, A, 5)
    assert (P.to_bytes_folded() == A.to_bytes_folded()[:9]).all()
    with pytest.raises(ft.FtError) as e:
        ft.Array.init_point(3, A, 77)
    assert e.value.code == 4
    assert len(ft.Array.from_scalars(np.zeros((0, 32), np.uint8))) == 0


def test_gather_scatter_delete(ft, orc):
    g = synth.rng(10)
    a = rand_points(orc, g, 50)
    ea = orc.encode(a)
    A = upload(ft, a)
    idx = [3, 0, 49, 3, 17]
    assert (A.get_subset(idx).to_bytes_folded() == ea[idx]).all()
    assert (A.get_range(5, 40, 7).to_bytes_folded() == ea[5:40:7][: (40 - 5) // 7]).all()
    with pytest.raises(ft.FtError) as e:
        A.get_subset([50])
    assert e.value.code == 4
    B = upload(ft, a)
    src = upload(ft, a[:3])
    B.assign_to_subset([10, 20, 30], src)
    want = ea.copy()
    want[[10, 20, 30]] = ea[:3]
    assert (B.to_bytes_folded() == want).all()
    B.assign_zero_to_subset([1, 2])
    want[[1, 2]] = orc.encode(orc.zeros(1))[0]
    assert (B.to_bytes_folded() == want).all()
    C = upload(ft, a)
    C.assign_to_range(4, 20, 5, upload(ft, a[40:44]))
    want = ea.copy()
    want[[4, 9, 14, 19]] = ea[40:44]
    assert (C.to_bytes_folded() == want).all()
    # a step past the range writes the first point only (no overflow in the count)
    C.assign_to_range(7, 9, 2**64 - 1, upload(ft, a[45:47]))
    want[7] = ea[45]
    assert (C.to_bytes_folded() == want).all()
    D = upload(ft, a)
    D.delete_subset([5, 5, 0, 49, 100])
    keep = [i for i in range(50) if i not in (0, 5, 49)]
    assert (D.to_bytes_folded() == ea[keep]).all()
    E = upload(ft, a)
    E.delete_range(10, 30, 3)
    keep = [i for i in range(50) if not (10 <= i < 30 and (i - 10) % 3 == 0)]
    assert (E.to_bytes_folded() == ea[keep]).all()


def test_set_length_mux_compare(ft, orc):
    g = synth.rng(11)
    a = rand_points(orc, g, 40)
    b = rand_points(orc, g, 40)
    ea, eb = orc.encode(a), orc.encode(b)
    zero = orc.encode(orc.zeros(1))[0]
    A = upload(ft, a)
    A.set_length(30)
    A.set_length(35)  # within the reserve: zero-extended
    assert (A.to_bytes_folded() == np.concatenate([ea[:30], np.tile(zero, (5, 1))])).all()
    A.set_length(10)  # at most half: reallocated
    A.set_length(12)
    assert (A.to_bytes_folded() == np.concatenate([ea[:10], np.tile(zero, (2, 1))])).all()
    # lengths whose byte sizes overflow are refused before any allocation
    for bad in (lambda: A.set_length(2**60), lambda: ft.Array.init_scalar(2**60)):
        with pytest.raises(ft.FtError) as e:
            bad()
        assert e.value.code == 1
    assert len(A) == 12
    cond = g.integers(0, 2, 40).astype(np.int64)
    M = upload(ft, a)
    M.mux(cond, upload(ft, b))
    assert (M.to_bytes_folded() == np.where(cond[:, None] != 0, ea, eb)).all()
    c = a.copy()
    c[::3] = b[::3]
    eq = upload(ft, a).equal(upload(ft, c))
    assert (eq == orc.equal(a, c)).all() and eq.sum() == 40 - len(range(0, 40, 3))
    assert (upload(ft, a).not_equal(upload(ft, c)) == 1 - eq).all()
    z = a.copy()
    z[[2, 7]] = orc.zeros(2)
    assert (upload(ft, z).index() == orc.index(z)).all()


@pytest.mark.parametrize("n", [0, 1, 2, 3, 127, 128, 129, 1023, 1024, 1025, 5000, 70001])
def test_reduce_scan_prescan(ft, orc, n):
    g = synth.rng(200 + n)
    a = rand_points(orc, g, n)
    A = upload(ft, a)
    A.reduce()
    assert len(A) == 1
    assert (A.to_bytes_folded() == orc.encode(orc.reduce(a, threads=8))).all()
    S = upload(ft, a)
    S.scan()
    assert (S.to_bytes_folded() == orc.encode(orc.scan(a))).all()
    X = upload(ft, a)
    X.prescan()
    assert (X.to_bytes_folded() == orc.encode(orc.scan(a, exclusive=True))).all()


@pytest.mark.parametrize("n", [262145, 300001])
def test_scan_large_by_linearity(ft, n):
    # sizes whose top level takes 16 points per thread: the scan of k_i * B
    # is (k_0 + ... + k_i) * B, computed by the comb from the prefix sums
    g = synth.rng(300 + n)
    k = g.integers(0, 1 << 20, n).astype(np.uint64)
    S = ft.Array.from_small_scalars(k)
    S.scan()
    assert (S.to_bytes_folded() == ft.Array.from_small_scalars(np.cumsum(k)).to_bytes_folded()).all()
    X = ft.Array.from_small_scalars(k)
    X.prescan()
    ex = np.concatenate([[0], np.cumsum(k)[:-1]]).astype(np.uint64)
    assert (X.to_bytes_folded() == ft.Array.from_small_scalars(ex).to_bytes_folded()).all()


@pytest.mark.parametrize("n,nseg", [(1, 1), (10, 10), (100, 1), (1000, 63), (20000, 1250), (70000, 2000)])
def test_segmented_sum_csr(ft, orc, n, nseg):
    g = synth.rng(300 + n)
    a = rand_points(orc, g, n)
    off = synth.csr_offsets(g, n, nseg)
    out = ft.segmented_sum_csr(off, upload(ft, a))
    assert (out.to_bytes_folded() == orc.encode(orc.segsum_csr(off, a, threads=8))).all()


def test_segmented_sum_empty_and_giant_segments(ft, orc):
    g = synth.rng(12)
    a = rand_points(orc, g, 9000)
    off = np.array([0, 0, 3, 3, 3, 8000, 8001, 8001, 9000, 9000], dtype=np.int32)
    out = ft.segmented_sum_csr(off, upload(ft, a))
    assert (out.to_bytes_folded() == orc.encode(orc.segsum_csr(off, a))).all()
    with pytest.raises(ft.FtError) as e:
        ft.segmented_sum_csr(np.array([0, 5, 3, 9000], np.int32), upload(ft, a))
    assert e.value.code == 3


def test_segmented_sum_long_segments_both_paths(ft, orc):
    """Long segments: the host-offsets call sums the layout through one scan
    and a difference of two prefixes per segment, the device-offsets call
    through the walk, whose join adds the thread parts of a long segment in
    turn; both equal the oracle, with empty segments at both ends and in the
    middle."""
    torch = pytest.importorskip("torch")
    g = synth.rng(14)
    n = 50000
    a = rand_points(orc, g, n)
    off = np.array([0, 0, 1, 20000, 20000, 20001, 45000, 49999, 50000, 50000], np.int32)
    want = orc.encode(orc.segsum_csr(off, a, threads=8))
    A = upload(ft, a)
    assert (ft.segmented_sum_csr(off, A).to_bytes_folded() == want).all()
    d_off = torch.from_numpy(off).cuda()
    torch.cuda.synchronize()
    out = ft.Array.init_scalar(len(off) - 1)
    ft.segmented_sum_csr_device(out, d_off.data_ptr(), len(off) - 1, A)
    assert (out.to_bytes_folded() == want).all()


@pytest.mark.parametrize("n,nseg", [(1, 1), (1000, 63), (70000, 2000), (300001, 20000)])
def test_ct_segmented_sum_both_halves(ft, orc, n, nseg):
    """Both halves of a ciphertext array summed over the same device offsets
    in one set of launches equal the oracle's segment sums of each half, with
    empty segments in the layout; outputs that alias the other half's input
    take the two single-array calls in order."""
    torch = pytest.importorskip("torch")
    g = synth.rng(700 + n)
    a1, a2 = rand_points(orc, g, n), rand_points(orc, g, n)
    off = synth.csr_offsets(g, n, nseg)
    if nseg > 2:
        off[1] = off[0]  # an empty first segment
        off[-2] = off[-1]  # and an empty last one
    w1 = orc.encode(orc.segsum_csr(off, a1, threads=8))
    w2 = orc.encode(orc.segsum_csr(off, a2, threads=8))
    d_off = torch.from_numpy(off).cuda()
    torch.cuda.synchronize()
    C1, C2 = upload(ft, a1), upload(ft, a2)
    o1, o2 = ft.Array.init_scalar(nseg), ft.Array.init_scalar(nseg)
    ft.ct_segmented_sum_csr_device(o1, o2, d_off.data_ptr(), nseg, C1, C2)
    assert (o1.to_bytes_folded() == w1).all()
    assert (o2.to_bytes_folded() == w2).all()
    if n == nseg:
        # one point a segment, out1 = c2: the two sums in order, the second
        # reading the first's result (each sum the identity map here)
        ft.ct_segmented_sum_csr_device(C2, o2, d_off.data_ptr(), nseg, C1, C2)
        assert (C2.to_bytes_folded() == w1).all()
        assert (o2.to_bytes_folded() == w1).all()
    with pytest.raises(ft.FtError) as e:
        ft.ct_segmented_sum_csr_device(o1, ft.Array.init_scalar(nseg + 1), d_off.data_ptr(), nseg, C1, C2)
    assert e.value.code == 2


def test_ct_segmented_sum_without_points(ft, orc):
    """Empty halves: every segment empty (the identity in both outputs, over
    whatever they held), and no segments at all (nothing written)."""
    torch = pytest.importorskip("torch")
    d_off = torch.zeros(4, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    g = synth.rng(19)
    o1, o2 = upload(ft, rand_points(orc, g, 3)), upload(ft, rand_points(orc, g, 3))
    e1, e2 = ft.Array.init_scalar(0), ft.Array.init_scalar(0)
    ft.ct_segmented_sum_csr_device(o1, o2, d_off.data_ptr(), 3, e1, e2)
    ident = ft.Array.init_scalar(3).to_bytes_folded()
    assert (o1.to_bytes_folded() == ident).all()
    assert (o2.to_bytes_folded() == ident).all()
    z1, z2 = ft.Array.init_scalar(0), ft.Array.init_scalar(0)
    ft.ct_segmented_sum_csr_device(z1, z2, d_off.data_ptr(), 0, e1, e2)
    assert len(z1) == 0 and len(z2) == 0


@pytest.mark.parametrize("n", [1, 2, 1000, 1 << 20])
def test_reduce_isum_all_keys_equal(ft, orc, n):
    """Every key the same (one segment of n points, a full reduction) and
    two keys splitting the points unevenly, accumulated into res."""
    g = synth.rng(500 + n)
    src = rand_points(orc, g, min(n, 4096))
    src = np.tile(src, (n // src.shape[0] + 1, 1))[:n].copy()
    res = rand_points(orc, g, 5)
    R = upload(ft, res)
    R.reduce_isum(np.full(n, 3, np.uint64), upload(ft, src))
    want = res.copy()
    want[3] = orc.add(res[3:4], orc.reduce(src, threads=8))[0]
    assert (R.to_bytes_folded() == orc.encode(want)).all()
    keys = np.where(np.arange(n) % 97 == 5, 0, 4).astype(np.uint64)
    R = upload(ft, res)
    R.reduce_isum(keys, upload(ft, src))
    w2, err = orc.isum(res, keys, src) if n <= 1000 else (None, 0)
    if w2 is None:
        w2 = res.copy()
        w2[0] = orc.add(res[0:1], orc.reduce(src[keys == 0], threads=8))[0]
        w2[4] = orc.add(res[4:5], orc.reduce(src[keys == 4], threads=8))[0]
    assert err == 0
    assert (R.to_bytes_folded() == orc.encode(w2)).all()


@pytest.mark.parametrize("n", [0, 1, 5, 1000, 1025, 70001])
@pytest.mark.parametrize("exclusive", [False, True])
def test_ct_scan(ft, orc, n, exclusive):
    """ftx_ct_scan: both halves in one call equal two ft_array_scan /
    ft_array_prescan calls and the oracle; the same array passed twice is
    scanned twice."""
    g = synth.rng(600 + n)
    a, b = rand_points(orc, g, n), rand_points(orc, g, n)
    A, B = upload(ft, a), upload(ft, b)
    ft.ct_scan(A, B, exclusive)
    assert (A.to_bytes_folded() == orc.encode(orc.scan(a, exclusive))).all()
    assert (B.to_bytes_folded() == orc.encode(orc.scan(b, exclusive))).all()
    C = upload(ft, a)
    ft.ct_scan(C, C, exclusive)
    assert (C.to_bytes_folded() == orc.encode(orc.scan(orc.scan(a, exclusive), exclusive))).all()
    if n:
        with pytest.raises(ft.FtError) as e:
            ft.ct_scan(upload(ft, a), upload(ft, b[:-1]))
        assert e.value.code == 2


@pytest.mark.parametrize("n,nres", [(1, 1), (50, 7), (3000, 100), (40000, 5000)])
def test_reduce_isum(ft, orc, n, nres):
    g = synth.rng(400 + n)
    src = rand_points(orc, g, n)
    res = rand_points(orc, g, nres)
    keys = g.integers(0, nres, n).astype(np.uint64)
    R = upload(ft, res)
    R.reduce_isum(keys, upload(ft, src))
    want, err = orc.isum(res, keys, src)
    assert err == 0
    assert (R.to_bytes_folded() == orc.encode(want)).all()
    with pytest.raises(ft.FtError) as e:
        R.reduce_isum(np.full(n, nres, np.uint64), upload(ft, src))
    assert e.value.code == 4
    assert (R.to_bytes_folded() == orc.encode(want)).all()  # unchanged on error


def test_wire_formats_vs_oracle(ft, orc):
    g = synth.rng(13)
    a = rand_points(orc, g, 1001)
    k = synth.scalars_mod_L(g, 1001)
    a = orc.mul(a, k, threads=8)  # non-trivial Z
    A = upload(ft, a)
    assert (A.to_bytes_folded() == orc.encode(a)).all()
    assert (A.to_bytes_affine() == orc.to_affine(a)).all()
    assert (A.to_bytes() == orc.to_ref160(a)).all()
    B, bad = ft.Array.from_bytes_folded(orc.encode(a))
    assert bad == -1
    assert (B.to_packed() == orc.decode(orc.encode(a))[0]).all()
    junk = g.integers(0, 256, (500, 32), dtype=np.uint8)
    J, jb = ft.Array.from_bytes_folded(junk)
    od, ob = orc.decode(junk)
    assert jb == ob
    assert (J.to_bytes_folded() == orc.encode(od)).all()
    assert J.validate() == orc.validate(od)
    with pytest.raises(ft.FtError) as e:
        ft.Array.from_bytes_folded(np.zeros(33, np.uint8))
    assert e.value.code == 3
    # a zero Z encodes like the reference (inverse of 0 is 0)
    zz = a[:9].copy()
    zz[4, 64:96] = 0
    assert (upload(ft, zz).to_bytes_folded() == orc.encode(zz)).all()
    assert (upload(ft, zz).to_bytes_affine() == orc.to_affine(zz)).all()


def test_encrypt_vs_oracle_and_decrypt(ft, orc):
    g = synth.rng(14)
    sk = synth.scalars_mod_L(g, 1)
    pk = orc.encode(orc.from_scalars(sk))[0]
    n = 600
    m = synth.plaintexts(g, n, 255)
    r = synth.scalars_mod_L(g, n)
    c1, c2 = ft.encrypt(pk, m, r, 8)
    o1, o2 = orc.encrypt(pk, m, r, threads=8)
    assert (c1.to_bytes_folded() == orc.encode(o1)).all()
    assert (c2.to_bytes_folded() == orc.encode(o2)).all()
    # decrypt: c2 - sk*c1 == m*B
    c1.scale(sk[0])
    c2.sub(c1)
    assert (c2.to_bytes_folded() == orc.encode(orc.from_scalars(orc.small_to_scalars(m)))).all()
    cand = g.integers(0, 256, (64, 32), dtype=np.uint8)
    bad_pk = next(c for c in cand if orc.decode(c[None])[1] == 0)  # an encoding the reference rejects
    with pytest.raises(ft.FtError) as e:
        ft.encrypt(bad_pk, m[:2], r[:2], 8)
    assert e.value.code == 5
