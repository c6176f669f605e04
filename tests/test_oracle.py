"""The oracle (oracle/ftoracle.c) against golden vectors from the reference's
own arithmetic, against the reference built here (when present) and against
libsodium through PyNaCl (when installed)."""
import numpy as np
import pytest

from conftest import hx, hxs
from libftcrypto_gb300 import synth


def test_run_tests_cases(orc, golden):
    pts = orc.from_scalars(orc.small_to_scalars(range(9)))
    assert bytes(orc.encode(orc.reduce(pts))[0]).hex() == golden["reduce_0_8"]
    scan = orc.scan(orc.from_scalars(orc.small_to_scalars(range(7))))
    assert [bytes(e).hex() for e in orc.encode(scan)] == golden["scan_0_6"]
    ex = golden["isum_example"]
    res = orc.from_scalars(orc.small_to_scalars(ex["res"]))
    src = orc.from_scalars(orc.small_to_scalars(ex["src"]))
    out, err = orc.isum(res, ex["keys"], src)
    assert err == 0
    assert [bytes(e).hex() for e in orc.encode(out)] == ex["out"]
    five = orc.from_scalars(orc.small_to_scalars([5]))
    ten = orc.add(five, five)
    assert [int(orc.equal(five, five)[0]), int(orc.equal(five, ten)[0])] == golden["equal_example"] == [1, 0]
    assert bytes(orc.encode(orc.zeros(1))[0]).hex() == golden["identity"]


def test_scalarmult(orc, golden):
    cases = golden["smul"]
    pts, bad = orc.decode(hxs(c["point"] for c in cases))
    assert bad == -1
    out = orc.mul(pts, hxs(c["scalar"] for c in cases))
    assert [bytes(e).hex() for e in orc.encode(out)] == [c["out"] for c in cases]
    sb = golden["smul_base"]
    scal = hxs(c["scalar"] for c in sb)
    assert [bytes(e).hex() for e in orc.encode(orc.from_scalars(scal))] == [c["ladder"] for c in sb]
    assert [bytes(e).hex() for e in orc.encode(orc.from_scalars(scal, comb=True))] == [c["comb"] for c in sb]


def test_add_sub_neg(orc, golden):
    cs = golden["addsub"]
    a, _ = orc.decode(hxs(c["a"] for c in cs))
    b, _ = orc.decode(hxs(c["b"] for c in cs))
    assert [bytes(e).hex() for e in orc.encode(orc.add(a, b))] == [c["sum"] for c in cs]
    assert [bytes(e).hex() for e in orc.encode(orc.sub(a, b))] == [c["diff"] for c in cs]
    assert [bytes(e).hex() for e in orc.encode(orc.neg(a))] == [c["neg_a"] for c in cs]


def test_decode_including_rejected(orc, golden):
    cs = golden["decode"]
    pts, bad = orc.decode(hxs(c["in"] for c in cs))
    oks = [c["ok"] for c in cs]
    assert bad == max(i for i, o in enumerate(oks) if not o)
    assert [bytes(e).hex() for e in orc.encode(pts)] == [c["reenc"] for c in cs]
    for i, c in enumerate(cs):
        assert (orc.validate(pts[i:i + 1]) == -1) == bool(c["valid"])


def test_affine_raw_validate(orc, golden):
    af = golden["affine"]
    pts, _ = orc.decode(hxs(c["enc"] for c in af))
    assert [bytes(e).hex() for e in orc.to_affine(pts)] == [c["affine"] for c in af]
    back = orc.from_affine(orc.to_affine(pts))
    assert orc.validate(back) == -1
    raw = golden["raw160"]
    p = orc.from_ref160(hxs(c["raw"] for c in raw))
    assert [bytes(e).hex() for e in orc.encode(p)] == [c["enc"] for c in raw]
    q = golden["validate_neg_quirk"]
    assert (orc.validate(orc.from_ref160(hx(q["raw"])[None])) == -1) == bool(q["valid"])


def test_encrypt(orc, golden):
    e = golden["encrypt"]
    cs = e["cases"]
    c1, c2 = orc.encrypt(hx(e["pk"]), [c["m"] for c in cs], hxs(c["r"] for c in cs))
    assert [bytes(x).hex() for x in orc.encode(c1)] == [c["c1"] for c in cs]
    assert [bytes(x).hex() for x in orc.encode(c2)] == [c["c2"] for c in cs]


def test_oracle_threads_agree(orc):
    g = synth.rng(3)
    s = synth.scalars_mod_L(g, 37)
    p = orc.from_scalars(s, threads=1)
    assert (orc.from_scalars(s, threads=4) == p).all()
    assert (orc.encode(orc.reduce(p, threads=5)) == orc.encode(orc.reduce(p, threads=1))).all()
    off = synth.csr_offsets(g, 37, 9)
    seg = orc.segsum_csr(off, p, threads=3)
    ref = np.stack([orc.reduce(p[off[i]:off[i + 1]])[0] for i in range(9)])
    assert (orc.encode(seg) == orc.encode(ref)).all()


def test_against_reference_build(orc):
    ref = pytest.importorskip("oracle.ref")
    if not ref.available():
        pytest.skip("reference sources not present (oracle/_ref not built)")
    g = synth.rng(11)
    s = synth.scalars_mod_L(g, 40)
    p = orc.from_scalars(s)
    k = synth.scalars_mod_L(g, 40)
    m = orc.mul(p, k)
    for i in range(40):
        rp = ref.scalarmult(bytes(k[i]), ref.scalarmult(bytes(s[i]), ref.base()))
        assert rp.enc() == bytes(orc.encode(m[i:i + 1])[0])
        # the reference's own (non-canonical) limbs are ingested exactly
        back = orc.from_ref160(np.frombuffer(rp.raw(), dtype=np.uint8)[None].copy())
        assert bytes(orc.encode(back)[0]) == rp.enc()


def test_against_libsodium(orc):
    nb = pytest.importorskip("nacl.bindings")
    g = synth.rng(12)
    s = synth.scalars_mod_L(g, 20)
    s[0] = 0
    s[0, 0] = 1
    enc = orc.encode(orc.from_scalars(s))
    for i in range(20):
        assert nb.crypto_scalarmult_ed25519_base_noclamp(bytes(s[i])) == bytes(enc[i])
    a, b = enc[2], enc[3]
    s2 = orc.encode(orc.add(*(orc.decode(x[None])[0] for x in (a, b))))
    assert nb.crypto_core_ed25519_add(bytes(a), bytes(b)) == bytes(s2[0])


def test_encode_mt_equals_encode(orc, golden):
    """The batched-inversion encoder used for the full-size configuration
    checks gives fto_encode's bytes: on-curve points, rejected decodes (off
    the curve), zero Z and ragged batch edges (n not a multiple of 64)."""
    g = synth.rng(13)
    on = orc.from_scalars(synth.scalars_mod_L(g, 150), threads=4)
    off, _ = orc.decode(hxs(c["in"] for c in golden["decode"]))
    zz = on[:5].copy()
    zz[:, 64:96] = 0                      # Z = 0
    zz[1, 64:96] = 0xff                   # Z = 2^256 - 1 (not zero mod p)
    zz[2, 64:96] = np.frombuffer(((1 << 255) - 19).to_bytes(32, "little"), dtype=np.uint8)  # Z = p
    pts = np.concatenate([on, off, zz, on[::-1]])
    want = orc.encode(pts)
    for threads in (1, 2, 3, 16):
        got = np.zeros_like(want)
        orc.lib().fto_encode_mt(orc._p(got), orc._p(pts), pts.shape[0], threads)
        assert (got == want).all()
    assert (orc.encode(pts, threads=5) == want).all()


@pytest.mark.parametrize("k", [0, 1, 2, 3, 1000, 65535, (1 << 32) - 1, (1 << 64) - 1])
def test_scale_u64_equals_ladder(orc, k):
    """Double-and-add by a public 64-bit k gives the reference ladder's group
    element (the oracle's fto_scale, sodium_ge.cu:650-731)."""
    g = synth.rng(14)
    pts = orc.from_scalars(synth.scalars_mod_L(g, 21), threads=4)
    want = orc.encode(orc.scale(pts, orc.small_to_scalars([k])[0]))
    assert (orc.encode(orc.scale_u64(pts, k, threads=3)) == want).all()
    ks = np.full(pts.shape[0], k, dtype=np.uint64)
    ks[::2] = 7
    each = orc.encode(orc.scale_u64_each(pts, ks, threads=4))
    assert (each[1::2] == want[1::2]).all()
    assert (each[::2] == orc.encode(orc.scale_u64(pts[::2], 7))).all()


@pytest.mark.parametrize("exclusive", [False, True])
def test_scan_mt_equals_serial_scan(orc, exclusive):
    g = synth.rng(15)
    pts = orc.from_scalars(synth.scalars_mod_L(g, 77), threads=4)
    want = orc.encode(orc.scan(pts, exclusive))
    for threads in (2, 5, 16, 100):
        assert (orc.encode(orc.scan(pts, exclusive, threads=threads)) == want).all()
