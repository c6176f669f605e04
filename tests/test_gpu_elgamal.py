"""ElGamal helpers beyond the reference's interface (ftx_rerandomise,
ftx_decrypt): decryption recovers the plaintexts through the device table of
j*B, re-randomisation adds exactly (r*B, r*PK) (checked against the oracle)
and leaves the plaintexts unchanged."""
import numpy as np
import pytest

from libftcrypto_gb300 import synth

pytestmark = pytest.mark.gpu


def keys(ft, g):
    sk = synth.scalars_mod_L(g, 1)
    pk_arr = ft.Array.from_scalars(sk)
    return sk[0], pk_arr.to_bytes_folded()[0], pk_arr.to_packed()


@pytest.mark.parametrize("n", [0, 1, 257, 3000])
def test_decrypt_roundtrip(ft, n):
    g = synth.rng(70 + n)
    sk, pk, _ = keys(ft, g)
    m = g.integers(0, 1000, size=n, dtype=np.uint64)
    if n >= 2:
        m[0], m[1] = 0, 999
    c1, c2 = ft.encrypt(pk, m, synth.scalars_mod_L(g, n), 10)
    assert (ft.decrypt(c1, c2, sk, 1000) == m).all()


def test_decrypt_out_of_range_wrong_key_and_sums(ft):
    g = synth.rng(81)
    sk, pk, _ = keys(ft, g)
    m = np.array([0, 5, 999, 1000, 1001, 4095], dtype=np.uint64)
    c1, c2 = ft.encrypt(pk, m, synth.scalars_mod_L(g, m.size), 12)
    got = ft.decrypt(c1, c2, sk, 1000)
    assert (got[:3] == m[:3]).all() and (got[3:] == ft.NO_PLAINTEXT).all()
    other, _, _ = keys(ft, g)  # c2 - sk'*c1 = m*B + r*(sk - sk')*B: no small plaintext
    assert (ft.decrypt(c1, c2, other, 1000) == ft.NO_PLAINTEXT).all()
    # a smaller table (rebuilt), then the homomorphic sum under a larger one
    assert (ft.decrypt(c1, c2, sk, 6)[:2] == m[:2]).all()
    assert (ft.decrypt(c1, c2, sk, 6)[2:] == ft.NO_PLAINTEXT).all()
    d1, d2 = ft.encrypt(pk, m, synth.scalars_mod_L(g, m.size), 12)
    c1.add(d1)
    c2.add(d2)
    assert (ft.decrypt(c1, c2, sk, 8192) == 2 * m).all()
    assert (ft.decrypt(c1, c2, sk, 1) == np.where(m == 0, 0, ft.NO_PLAINTEXT)).all()


def test_decrypt_arguments(ft):
    g = synth.rng(82)
    sk, pk, _ = keys(ft, g)
    c1, c2 = ft.encrypt(pk, np.zeros(4, np.uint64), synth.scalars_mod_L(g, 4), 1)
    for bad in (0, ft.DECRYPT_MAX_M + 1):
        with pytest.raises(ft.FtError) as e:
            ft.decrypt(c1, c2, sk, bad)
        assert e.value.code == 3
    with pytest.raises(ft.FtError) as e:
        ft.decrypt(c1, c2.get_range(0, 3, 1), sk, 10)
    assert e.value.code == 2


def test_rerandomise_device_matches_host(ft):
    torch = pytest.importorskip("torch")
    g = synth.rng(88)
    sk, pk, _ = keys(ft, g)
    m = g.integers(0, 4, size=700, dtype=np.uint64)
    r1, r2 = synth.scalars_mod_L(g, 700), synth.scalars_mod_L(g, 700)
    a1, a2 = ft.encrypt(pk, m, r1, 2)
    b1, b2 = ft.encrypt(pk, m, r1, 2)
    ft.rerandomise(a1, a2, pk, r2)
    d_r = torch.from_numpy(r2).cuda()
    torch.cuda.synchronize()
    ft.rerandomise_device(b1, b2, pk, d_r.data_ptr(), 700)
    assert (a1.to_bytes_folded() == b1.to_bytes_folded()).all()
    assert (a2.to_bytes_folded() == b2.to_bytes_folded()).all()
    assert (ft.decrypt(b1, b2, sk, 4) == m).all()


def test_rerandomise_empty(ft):
    g = synth.rng(89)
    _, pk, _ = keys(ft, g)
    c1, c2 = ft.Array.init_scalar(0), ft.Array.init_scalar(0)
    ft.rerandomise(c1, c2, pk, synth.scalars_mod_L(g, 0))
    assert len(c1) == 0 and len(c2) == 0


@pytest.mark.parametrize("n", [1, 300, 2049])
def test_rerandomise_vs_oracle(ft, orc, n):
    g = synth.rng(90 + n)
    sk, pk, pk_packed = keys(ft, g)
    m = g.integers(0, 256, size=n, dtype=np.uint64)
    c1, c2 = ft.encrypt(pk, m, synth.scalars_mod_L(g, n), 8)
    old1, old2 = c1.to_packed(), c2.to_packed()
    r2 = synth.scalars_mod_L(g, n)
    ft.rerandomise(c1, c2, pk, r2)
    want1 = orc.add(old1, orc.from_scalars(r2, threads=8))
    want2 = orc.add(old2, orc.mul(np.repeat(pk_packed, n, axis=0), r2, threads=8))
    assert (c1.to_bytes_folded() == orc.encode(want1)).all()
    assert (c2.to_bytes_folded() == orc.encode(want2)).all()
    assert (c1.to_bytes_folded() != orc.encode(old1)).any(axis=1).all()
    assert (ft.decrypt(c1, c2, sk, 256) == m).all()
    with pytest.raises(ft.FtError) as e:
        ft.rerandomise(c1, c2, pk, r2[: n - 1] if n > 1 else synth.scalars_mod_L(g, 2))
    assert e.value.code == 2


@pytest.mark.parametrize("n", [0, 1, 1000])
def test_ct_add_sub_match_ft_add(ft, orc, n):
    """ftx_ct_add / ftx_ct_sub (one launch over both halves) equal ft_add /
    ft_sub on each half, also when arrays alias."""
    g = synth.rng(110 + n)
    pts = [orc.from_scalars(synth.scalars_mod_L(g, n), threads=8) for _ in range(4)]

    def arrs():
        return [ft.Array.from_packed(p) for p in pts]

    for op in ("add", "sub"):
        fn = ft.ct_add if op == "add" else ft.ct_sub
        for case in ("plain", "d1_is_c1", "d2_is_c1", "c1_is_c2"):
            c1, c2, d1, d2 = arrs()
            e1, e2, f1, f2 = arrs()
            if case == "d1_is_c1":
                d1, f1 = c1, e1
            elif case == "d2_is_c1":
                d2, f2 = c1, e1
            elif case == "c1_is_c2":
                c2, e2 = c1, e1
            fn(c1, c2, d1, d2)
            getattr(e1, op)(f1)
            getattr(e2, op)(f2)
            assert (c1.to_packed() == e1.to_packed()).all(), (op, case)
            assert (c2.to_packed() == e2.to_packed()).all(), (op, case)
    if n:
        c1, c2, d1, d2 = arrs()
        with pytest.raises(ft.FtError) as e:
            ft.ct_add(c1, c2, d1.get_range(0, n - 1, 1) if n > 1 else ft.Array.init_scalar(2), d2)
        assert e.value.code == 2


def test_encrypt_with_alternating_keys(ft, orc):
    # more keys than the library caches key tables for, used in turn and
    # again: each encryption equals the oracle's under its own key
    g = synth.rng(77)
    ks = [synth.scalars_mod_L(g, 1) for _ in range(6)]
    pks = [orc.encode(orc.from_scalars(sk))[0] for sk in ks]
    n = 33
    for rnd in range(2):
        for j in (0, 1, 2, 3, 4, 5, 1, 0):
            m = synth.plaintexts(g, n, 255)
            r = synth.scalars_mod_L(g, n)
            c1, c2 = ft.encrypt(pks[j], m, r, 8)
            o1, o2 = orc.encrypt(pks[j], m, r)
            assert (c1.to_bytes_folded() == orc.encode(o1)).all()
            assert (c2.to_bytes_folded() == orc.encode(o2)).all(), (rnd, j)


@pytest.mark.parametrize("n", [1, 1000, 100001])
def test_encrypt_and_rerandomise_halves(ft, orc, n):
    """The encryption kernel computes c1 and c2 as separate work units (spread
    over the grid) unless both are one array, in which case each thread does
    c1's half, then c2's, as one call to each would: encrypting into one array
    twice leaves c2's value, re-randomising it adds r*B then r*PK."""
    torch = pytest.importorskip("torch")
    g = synth.rng(140 + n)
    sk, pk, pk_packed = keys(ft, g)
    m = g.integers(0, 256, size=n, dtype=np.uint64)
    r = synth.scalars_mod_L(g, n)
    d_m = torch.from_numpy(m.view(np.int64)).cuda()
    d_r = torch.from_numpy(r).cuda()
    torch.cuda.synchronize()
    rB = orc.from_scalars(r, threads=8)
    rPK = orc.mul(np.repeat(pk_packed, n, axis=0), r, threads=8)
    c2_want = orc.add(rPK, orc.from_scalars(orc.small_to_scalars(m), threads=8), threads=8)
    # separate arrays: both halves as separate units
    c1, c2 = ft.Array.init_scalar(n), ft.Array.init_scalar(n)
    ft.encrypt_device(c1, c2, pk, d_m.data_ptr(), d_r.data_ptr(), n, 8)
    assert (c1.to_bytes_folded() == orc.encode(rB, 8)).all()
    assert (c2.to_bytes_folded() == orc.encode(c2_want, 8)).all()
    # one array for both: c2's value wins, as with the halves in order
    c = ft.Array.init_scalar(n)
    ft.encrypt_device(c, c, pk, d_m.data_ptr(), d_r.data_ptr(), n, 8)
    assert (c.to_bytes_folded() == orc.encode(c2_want, 8)).all()
    # re-randomising one array as both halves adds r*B and r*PK
    r2 = synth.scalars_mod_L(g, n)
    before = c.to_packed()
    ft.rerandomise(c, c, pk, r2)
    want = orc.add(orc.add(before, orc.from_scalars(r2, threads=8), threads=8),
                   orc.mul(np.repeat(pk_packed, n, axis=0), r2, threads=8), threads=8)
    assert (c.to_bytes_folded() == orc.encode(want, 8)).all()


@pytest.mark.parametrize("n", [1, 38912, 100001])
def test_encrypt_host_inputs_in_two_parts(ft, orc, n):
    """ftx_encrypt copies its host inputs in two parts (the first, one pass of
    the encryption grid — 38,912 ciphertexts at 152 SMs — encrypted while the
    rest is copied) and checks the plaintext bound on the device.  The points
    equal ftx_encrypt_device's on the same inputs, from pinned and from
    pageable buffers, and the oracle's on a sample; a plaintext at 2^bits in
    the first part, the middle or the last element fails the call with
    FT_ERR_BAD_SIZE; with 64-bit plaintexts nothing is rejected."""
    torch = pytest.importorskip("torch")
    g = synth.rng(170 + n)
    sk, pk, pk_packed = keys(ft, g)
    m = g.integers(0, 1 << 12, size=n, dtype=np.uint64)
    r = synth.scalars_mod_L(g, n)

    def on_device(mm, bits):
        d_m, d_r = torch.from_numpy(mm.view(np.int64)).cuda(), torch.from_numpy(r).cuda()
        torch.cuda.synchronize()
        w1, w2 = ft.Array.init_scalar(n), ft.Array.init_scalar(n)
        ft.encrypt_device(w1, w2, pk, d_m.data_ptr(), d_r.data_ptr(), n, bits)
        return w1.to_bytes_folded(), w2.to_bytes_folded()

    want1, want2 = on_device(m, 12)
    idx = np.unique(np.concatenate([[0, n - 1], g.integers(0, n, 64)]))
    rs = r[idx]
    rB = orc.from_scalars(rs, threads=8)
    c2_want = orc.add(orc.mul(np.repeat(pk_packed, len(idx), axis=0), rs, threads=8),
                      orc.from_scalars(orc.small_to_scalars(m[idx]), threads=8), threads=8)
    assert (want1[idx] == orc.encode(rB)).all()
    assert (want2[idx] == orc.encode(c2_want)).all()
    hm_t = torch.from_numpy(m.view(np.int64)).pin_memory()
    hr_t = torch.from_numpy(r).pin_memory()
    for mm, rr in ((hm_t.numpy().view(np.uint64), hr_t.numpy()), (m, r)):
        c1, c2 = ft.encrypt(pk, mm, rr, 12)
        assert (c1.to_bytes_folded() == want1).all()
        assert (c2.to_bytes_folded() == want2).all()
    for pos in sorted({0, n // 2, n - 1}):
        bad = m.copy()
        bad[pos] = 1 << 12
        with pytest.raises(ft.FtError) as e:
            ft.encrypt(pk, bad, r, 12)
        assert e.value.code == 3
    big = m | np.uint64(1 << 63)
    w1, w2 = on_device(big, 64)
    c1, c2 = ft.encrypt(pk, big, r, 64)
    assert (c1.to_bytes_folded() == w1).all()
    assert (c2.to_bytes_folded() == w2).all()
