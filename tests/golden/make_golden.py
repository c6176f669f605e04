"""Generate tests/golden/golden.json from the reference's own arithmetic.

Runs oracle/_ref/libftref.so (the reference's sodium_fe.cu / sodium_ge.cu
compiled for the host by oracle/build_ref.sh; needs the reference source
tree) and records folded encodings for:
  * run_tests.cc's cases (reduce of 0..8, scan of 0..6, the ft_reduce_isum
    example, ft_equal and ft_array_contains), composed from the reference's
    per-point helpers with the semantics of ftcrypto.cu;
  * variable-base and fixed-base scalar multiplication, add, sub, the
    reference's ft_neg, decoding of random bytes (accepted and rejected),
    affine round trips, validation, raw 160-byte limb structs, and ElGamal
    encryption in the reference's composition.

Usage:  python tests/golden/make_golden.py   (writes golden.json beside it)
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), os.pardir, os.pardir))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import oracle.ref as ref  # noqa: E402
from libftcrypto_gb300 import synth  # noqa: E402

L = synth.L


def h(b: bytes) -> str:
    return bytes(b).hex()


def sc(v: int) -> bytes:
    return int(v % 2**256).to_bytes(32, "little")


def smul_b(v: int) -> ref.Pt:
    return ref.scalarmult(sc(v), ref.base())


def main():
    if not ref.available():
        oracle.build_ref()
    assert ref.available(), "oracle/_ref/libftref.so needs the reference sources"
    g = synth.rng(20240601)
    out = {"generator": "tests/golden/make_golden.py (reference sodium_fe.cu/sodium_ge.cu, host build)"}

    # --- run_tests.cc cases
    vals = [smul_b(i) for i in range(9)]
    acc = ref.zero()
    for p in vals:
        ref.addto(acc, p)
    out["reduce_0_8"] = h(acc.enc())  # run_tests.cc:121-126
    acc = ref.zero()
    scan = []
    for i in range(7):
        ref.addto(acc, smul_b(i))
        scan.append(h(acc.enc()))
    out["scan_0_6"] = scan  # run_tests.cc:128-134
    res = [smul_b(v) for v in (5, 8, 20, 30, 50)]
    src = [smul_b(v) for v in (10, 20, 30)]
    for k, p in zip((2, 2, 3), src):
        ref.addto(res[k], p)
    out["isum_example"] = {"res": [5, 8, 20, 30, 50], "keys": [2, 2, 3], "src": [10, 20, 30],
                           "out": [h(p.enc()) for p in res]}  # run_tests.cc:175-189
    five = smul_b(5)
    ten = smul_b(5)
    ref.addto(ten, five)
    out["equal_example"] = [ref.equal(smul_b(5), smul_b(5)), ref.equal(five, ten)]  # run_tests.cc:140-155
    arr = [smul_b(v) for v in range(1, 8)]
    probe = [smul_b(v) for v in (3, 5, 8, 2)]
    out["contains_example"] = [int(any(ref.equal(p, a) for a in arr)) for p in probe]  # run_tests.cc:157-172
    out["identity"] = h(ref.zero().enc())
    out["generator"] = h(ref.base().enc())

    # --- scalar multiplication
    edge = [0, 1, 2, 7, 8, 9, 15, 16, 17, 255, 256, L - 1, L, L + 1, 2**252, 2**253 - 1,
            2**255 - 19, 2**255 - 1, 2**255, 2**256 - 1]
    rnd = [synth.scalar_to_int(s) for s in synth.scalars_mod_L(g, 24)]
    scal = edge + rnd
    pts = [smul_b(synth.scalar_to_int(s)) for s in synth.scalars_mod_L(g, len(scal))]
    out["smul"] = [{"point": h(p.enc()), "scalar": h(sc(v)), "out": h(ref.scalarmult(sc(v), p).enc())}
                   for p, v in zip(pts, scal)]
    out["smul_base"] = [{"scalar": h(sc(v)), "ladder": h(smul_b(v).enc()),
                         "comb": h(ref.scalarmult_base(sc(v)).enc())} for v in scal]

    # --- add / sub / neg
    a = [smul_b(synth.scalar_to_int(s)) for s in synth.scalars_mod_L(g, 16)]
    b = [smul_b(synth.scalar_to_int(s)) for s in synth.scalars_mod_L(g, 16)]
    a[0] = ref.zero()
    b[1] = ref.zero()
    b[2] = a[2].copy()
    addv, subv, negv = [], [], []
    for x, y in zip(a, b):
        s = x.copy(); ref.addto(s, y)
        d = x.copy(); ref.subfrom(d, y)
        n = x.copy(); ref.neg(n)
        addv.append({"a": h(x.enc()), "b": h(y.enc()), "sum": h(s.enc()), "diff": h(d.enc()), "neg_a": h(n.enc())})
    out["addsub"] = addv

    # --- decoding, including rejected encodings (the stored point re-encoded)
    dec = []
    raw = [bytes(g.integers(0, 256, 32, dtype=np.uint8)) for _ in range(48)]
    raw += [bytes([0xff] * 31 + [0x7f]), bytes([0xec] + [0xff] * 30 + [0x7f]), bytes([0x01] + [0] * 30 + [0x80]),
            bytes(32), bytes([0] * 31 + [0x80])]
    for e in raw:
        p, r = ref.decode(e)
        dec.append({"in": h(e), "ok": int(r == 0), "reenc": h(p.enc()), "valid": ref.valid(p)})
    out["decode"] = dec

    # --- affine, validation and raw reference limbs
    aff = []
    for p in a[:8]:
        af = ref.to_affine(p)
        q = ref.from_affine(af)
        aff.append({"enc": h(p.enc()), "affine": h(af), "valid": ref.valid(q)})
    out["affine"] = aff
    out["raw160"] = [{"raw": h(p.raw()), "enc": h(p.enc())} for p in a[:8] + b[:8]]
    negp = a[5].copy()
    ref.neg(negp)
    out["validate_neg_quirk"] = {"raw": h(negp.raw()), "valid": ref.valid(negp)}

    # --- ElGamal encryption in the reference's composition
    sk = synth.scalar_to_int(synth.scalars_mod_L(g, 1)[0])
    pk = smul_b(sk)
    ms = [0, 1, 255, 7, 2**32 + 5, 2**64 - 1] + [int(x) for x in g.integers(0, 256, 10)]
    rs = [synth.scalar_to_int(s) for s in synth.scalars_mod_L(g, len(ms))]
    enc = []
    for m, r in zip(ms, rs):
        c1 = smul_b(r)
        c2 = smul_b(m)
        ref.addto(c2, ref.scalarmult(sc(r), pk))
        enc.append({"m": m, "r": h(sc(r)), "c1": h(c1.enc()), "c2": h(c2.enc())})
    out["encrypt"] = {"sk": h(sc(sk)), "pk": h(pk.enc()), "cases": enc}

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(path)


if __name__ == "__main__":
    main()
