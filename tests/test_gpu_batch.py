"""The batched form (ftx_batch_*: one persistent launch replayed from a CUDA
graph) gives exactly the results of the same operations called one array at
a time, and those match the oracle."""
import numpy as np
import pytest

from libftcrypto_gb300 import synth

pytestmark = pytest.mark.gpu


def make_arrays(ft, base, work, g):
    arrs = []
    for w in work:
        n = w["len"]
        c1 = base.get_subset(g.integers(0, len(base), n))
        c2 = base.get_subset(g.integers(0, len(base), n))
        extra = {}
        if w["op"] == "add":
            extra["s1"] = base.get_subset(g.integers(0, len(base), n))
            extra["s2"] = base.get_subset(g.integers(0, len(base), n))
        if w["op"] == "segsum":
            nseg = len(w["offsets"]) - 1
            extra["o1"] = ft.Array.init_scalar(nseg)
            extra["o2"] = ft.Array.init_scalar(nseg)
        arrs.append((c1, c2, extra))
    return arrs


def clone(ft, arrs):
    out = []
    for c1, c2, ex in arrs:
        out.append((c1.get_range(0, len(c1), 1), c2.get_range(0, len(c2), 1),
                    {k: v.get_range(0, len(v), 1) for k, v in ex.items()}))
    return out


def run_plain(ft, work, arrs):
    for w, (c1, c2, ex) in zip(work, arrs):
        if w["op"] == "add":
            c1.add(ex["s1"])
            c2.add(ex["s2"])
        elif w["op"] == "scale":
            c1.scale_small(w["k"], w["bits"])
            c2.scale_small(w["k"], w["bits"])
        else:
            ex["o1"].free()
            ex["o2"].free()
            ex["o1"] = ft.segmented_sum_csr(w["offsets"], c1)
            ex["o2"] = ft.segmented_sum_csr(w["offsets"], c2)


def build_batch(ft, work, arrs):
    b = ft.Batch()
    for w, (c1, c2, ex) in zip(work, arrs):
        if w["op"] == "add":
            b.add(c1, ex["s1"])
            b.add(c2, ex["s2"])
        elif w["op"] == "scale":
            b.scale_small(c1, w["k"], w["bits"])
            b.scale_small(c2, w["k"], w["bits"])
        else:
            b.segmented_sum(ex["o1"], w["offsets"], c1)
            b.segmented_sum(ex["o2"], w["offsets"], c2)
    return b


def outputs(work, arrs):
    res = []
    for w, (c1, c2, ex) in zip(work, arrs):
        if w["op"] == "segsum":
            res += [ex["o1"].to_bytes_folded(), ex["o2"].to_bytes_folded()]
        else:
            res += [c1.to_bytes_folded(), c2.to_bytes_folded()]
    return res


def test_batch_equals_plain_and_oracle(ft, orc):
    g = synth.rng(31)
    base = ft.Array.from_scalars(synth.scalars_mod_L(g, 512))
    work = synth.uneven_mix(g, n_arrays=48, max_len=3000)
    arrs = make_arrays(ft, base, work, g)
    i = next(j for j, w in enumerate(work) if w["op"] == "scale")
    scale_in = arrs[i][0].to_packed()
    plain = clone(ft, arrs)
    run_plain(ft, work, plain)
    b = build_batch(ft, work, arrs)
    items, ops = b.info()
    assert ops == 2 * len(work) and items >= ops
    b.run()
    got, want = outputs(work, arrs), outputs(work, plain)
    for x, y in zip(got, want):
        assert (x == y).all()
    # replaying the graph re-runs every operation: a second run equals the
    # plain calls applied twice (segmented sums read unchanged inputs)
    b.run()
    run_plain(ft, work, plain)
    for x, y in zip(outputs(work, arrs), outputs(work, plain)):
        assert (x == y).all()
    # one twice-scaled array against the oracle
    k = synth.int_to_scalar(work[i]["k"])
    want = orc.scale(orc.scale(scale_in, k, threads=8), k, threads=8)
    assert (arrs[i][0].to_bytes_folded() == orc.encode(want)).all()


def test_scale_small_matches_scale(ft, orc):
    g = synth.rng(32)
    # 300: one block with a partial warp; 1000: three blocks, a partial last one
    for n, ks in ((300, (0, 1, 7, 1000, 2**32 - 1)), (1000, (3, 2**31 + 5))):
        pts = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
        for k in ks:
            a = ft.Array.from_packed(pts)
            a.scale_small(k)
            want = orc.scale(pts, synth.int_to_scalar(k), threads=8)
            assert (a.to_bytes_folded() == orc.encode(want)).all(), (n, k)


@pytest.mark.parametrize("width", [2, 3, 4])
def test_scale_bounded_windows(ft, orc, width):
    """ftx_scale_bounded at each window width: exact at the largest k of each
    bound, and in the batched form; k >= 2^bits and bits outside 1..32 are
    refused."""
    g = synth.rng(33 + width)
    pts = orc.from_scalars(synth.scalars_mod_L(g, 500), threads=8)
    before = ft.tune_get(ft.TUNE_SCALE_WINDOW)
    ft.tune(ft.TUNE_SCALE_WINDOW, width)
    for bits in (1, 3, 7, 10, 11, 16, 31, 32):
        for k in {(1 << bits) - 1, (1 << bits) // 2, 1}:
            a = ft.Array.from_packed(pts)
            a.scale_small(k, bits)
            want = orc.encode(orc.scale(pts, synth.int_to_scalar(k), threads=8))
            assert (a.to_bytes_folded() == want).all(), (bits, k)
            c = ft.Array.from_packed(pts)
            b = ft.Batch()
            b.scale_small(c, k, bits)
            b.run()
            assert (c.to_bytes_folded() == want).all(), (bits, k)
            b.free()
    ft.tune(ft.TUNE_SCALE_WINDOW, before)
    a = ft.Array.from_packed(pts[:4])
    for k, bits in ((1024, 10), (2, 1), (1, 0), (1, 33)):
        with pytest.raises(ft.FtError) as e:
            a.scale_small(k, bits)
        assert e.value.code == 3
    for bad in (1, 5):
        with pytest.raises(ft.FtError):
            ft.tune(ft.TUNE_SCALE_WINDOW, bad)


def test_scale_small_c_entry_points(ft, orc):
    """ftx_scale_small and ftx_batch_scale_small (the 32-bit bound) through
    the C ABI directly."""
    g = synth.rng(34)
    pts = orc.from_scalars(synth.scalars_mod_L(g, 100), threads=8)
    k = 2**32 - 3
    want = orc.encode(orc.scale(pts, synth.int_to_scalar(k), threads=8))
    L = ft.api.lib()
    a = ft.Array.from_packed(pts)
    ft.check(L.ftx_scale_small(a.handle, k))
    assert (a.to_bytes_folded() == want).all()
    a = ft.Array.from_packed(pts)
    b = ft.Batch()
    ft.check(L.ftx_batch_scale_small(b._h, a.handle, k))
    b._keep.append(a)
    b.run()
    assert (a.to_bytes_folded() == want).all()
    b.free()


def test_empty_batch_and_arrays(ft):
    """A batch with no operations, and operations on empty arrays, run and
    change nothing."""
    b = ft.Batch()
    b.run()
    b.run()
    b.free()
    e = ft.Array.init_scalar(0)
    e.scale_small(5, 3)
    b = ft.Batch()
    b.scale_small(e, 5, 3)
    b.add(ft.Array.init_scalar(0), ft.Array.init_scalar(0))
    b.run()
    b.free()
    assert len(e) == 0


def test_batch_rejects_conflicts(ft):
    g = synth.rng(33)
    a = ft.Array.from_scalars(synth.scalars_mod_L(g, 10))
    c = ft.Array.from_scalars(synth.scalars_mod_L(g, 10))
    b = ft.Batch()
    b.add(a, c)
    with pytest.raises(ft.FtError):
        b.scale_small(a, 3)  # a is already written by the batch
    with pytest.raises(ft.FtError):
        b.add(c, a)          # c is read, a is written
    b.run()
    with pytest.raises(ft.FtError):
        b.scale_small(ft.Array.from_scalars(synth.scalars_mod_L(g, 2)), 3)  # recorded after the first run


def test_batch_refuses_reallocated_arrays(ft, orc):
    g = synth.rng(34)
    sa, sc = synth.scalars_mod_L(g, 40), synth.scalars_mod_L(g, 40)
    a, c = ft.Array.from_scalars(sa), ft.Array.from_scalars(sc)
    b = ft.Batch()
    b.add(a, c)
    b.run()
    want = orc.encode(orc.add(orc.from_scalars(sa), orc.from_scalars(sc)))
    assert (a.to_bytes_folded() == want).all()
    a.set_length(10)  # at most half: new storage, which the work list does not know
    with pytest.raises(ft.FtError) as e:
        b.run()
    assert e.value.code == 2
    assert (a.to_bytes_folded() == want[:10]).all()  # nothing ran
