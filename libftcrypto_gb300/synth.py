"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The reference publishes no dataset; every input is drawn from
numpy.random.Generator(PCG64(seed)):
  * scalars uniform mod L = 2^252 + 27742317777372353535851937790883648493
    (253-bit rejection sampling), 32-byte little-endian;
  * a key pair: sk uniform mod L, pk = sk * B (computed by the caller);
  * plaintexts uniform in {0,1} or [0, 255];
  * CSR segment offsets whose lengths are the gaps between nseg-1 distinct
    uniform breakpoints in (0, n): every segment has length >= 1, the total
    is exactly n and lengths are close to geometric with mean n / nseg.
"""
from __future__ import annotations

import numpy as np

L = 2**252 + 27742317777372353535851937790883648493
_L_LIMBS = [(L >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(4)]


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _lt_L(c: np.ndarray) -> np.ndarray:
    l0, l1, l2, l3 = (np.uint64(x) for x in _L_LIMBS)
    c0, c1, c2, c3 = c[:, 0], c[:, 1], c[:, 2], c[:, 3]
    return (c3 < l3) | ((c3 == l3) & ((c2 < l2) | ((c2 == l2) & ((c1 < l1) | ((c1 == l1) & (c0 < l0))))))


def scalars_mod_L(g: np.random.Generator, n: int) -> np.ndarray:
    """(n, 32) uint8: uniform scalars in [0, L)."""
    out = np.empty((n, 4), dtype=np.uint64)
    filled = 0
    mask = np.uint64((1 << 61) - 1)  # 3*64 + 61 = 253 bits
    while filled < n:
        k = 2 * (n - filled) + 64
        cand = np.frombuffer(g.bytes(32 * k), dtype="<u8").reshape(k, 4).copy()
        cand[:, 3] &= mask
        ok = cand[_lt_L(cand)]
        take = min(len(ok), n - filled)
        out[filled:filled + take] = ok[:take]
        filled += take
    return out.view(np.uint8).reshape(n, 32).copy()


def scalar_to_int(s: np.ndarray) -> int:
    return int.from_bytes(bytes(np.asarray(s, dtype=np.uint8).reshape(32)), "little")


def int_to_scalar(v: int) -> np.ndarray:
    return np.frombuffer(int(v).to_bytes(32, "little"), dtype=np.uint8).copy()


def plaintexts(g: np.random.Generator, n: int, hi: int) -> np.ndarray:
    """(n,) uint64 uniform in [0, hi]."""
    return g.integers(0, hi + 1, size=n, dtype=np.uint64)


def csr_offsets(g: np.random.Generator, n: int, nseg: int) -> np.ndarray:
    """(nseg + 1,) int32 offsets of nseg non-empty segments covering n points."""
    if nseg < 1 or nseg > n:
        raise ValueError("need 1 <= nseg <= n")
    cuts = g.choice(n - 1, size=nseg - 1, replace=False, shuffle=False) + 1 if nseg > 1 else np.zeros(0, np.int64)
    cuts = np.sort(cuts.astype(np.int64))
    return np.concatenate([[0], cuts, [n]]).astype(np.int32)


def segment_ids(offsets: np.ndarray) -> np.ndarray:
    """Segment index of every point (the ft_reduce_isum keys of a CSR layout)."""
    lens = np.diff(offsets.astype(np.int64))
    return np.repeat(np.arange(len(lens), dtype=np.uint64), lens)


def uneven_mix(g: np.random.Generator, n_arrays: int = 4096, max_len: int = 65536, seg_mean: int = 8):
    """The uneven batched workload: n_arrays ciphertext arrays with lengths
    floor(exp(U(0, ln max_len))) clamped to [1, max_len], each drawing one op:
    add (40%), multiply by a scalar uniform in [1, 1000] (30%; "bits" = 10
    is the public bound k < 2^10 of that draw), or a segmented sum with
    ~geometric segments of mean seg_mean (30%).
    Returns a list of dicts {len, op, k and bits | offsets}."""
    lens = np.clip(np.floor(np.exp(g.uniform(0.0, np.log(max_len), n_arrays))), 1, max_len).astype(np.int64)
    ops = g.choice(3, size=n_arrays, p=[0.4, 0.3, 0.3])
    out = []
    for n, op in zip(lens, ops):
        n = int(n)
        if op == 0:
            out.append({"len": n, "op": "add"})
        elif op == 1:
            out.append({"len": n, "op": "scale", "k": int(g.integers(1, 1001)), "bits": 10})
        else:
            nseg = max(1, int(round(n / seg_mean)))
            out.append({"len": n, "op": "segsum", "offsets": csr_offsets(g, n, nseg)})
    return out
