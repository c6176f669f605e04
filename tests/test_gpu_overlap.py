"""Exports and scalar uploads that overlap queued work.

An export of an array whose last writer marked it (ft_mul, ftx_mul_device,
the encryptions) runs on the library's transfer stream after that writer
only, so it overlaps kernels queued later on the library stream; ft_mul
copies pinned host scalars through two staging buffers on that stream.
These tests check that the overlapped paths return the same bytes as the
ordered ones and as the oracle, and that every other use of an array in
between (an in-place operation, a batch run, a write through a device view)
sends its export back to stream order."""
import ctypes

import numpy as np
import pytest

from libftcrypto_gb300 import synth

pytestmark = pytest.mark.gpu


_PINNED = []  # the pinned tensors behind the arrays pinned() returns


def pinned(torch, a: np.ndarray) -> np.ndarray:
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    _PINNED.append(t)
    return t.numpy()


def raw(ft, arr, torch=None):
    """ft_array_to_bytes into pageable memory, or pinned memory with torch."""
    n = len(arr)
    if torch is None:
        out = np.zeros(n * 160, np.uint8)
    else:
        out = pinned(torch, np.zeros(n * 160, np.uint8))
    ft.check(ft.api.lib().ft_array_to_bytes(out.ctypes.data_as(ctypes.c_void_p), out.size, arr.handle))
    return np.array(out).reshape(n, 160)


def test_mul_then_export_while_next_mul_runs(ft, orc):
    """The e2e pattern: c1 *= k, c2 *= k (pinned scalars), then the exports of
    c1 (overlapping c2's ladder) and c2; bytes equal the oracle's, in the raw,
    folded, affine and packed formats, and equal a second, ordered export."""
    torch = pytest.importorskip("torch")
    g = synth.rng(71)
    n = 70001
    p1 = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    p2 = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    k = synth.scalars_mod_L(g, n)
    w1, w2 = orc.mul(p1, k, threads=8), orc.mul(p2, k, threads=8)
    c1, c2 = ft.Array.from_packed(p1), ft.Array.from_packed(p2)
    hk = pinned(torch, k)
    c1.mul(hk)
    c2.mul(hk)
    got1 = raw(ft, c1, torch)
    got2 = raw(ft, c2, torch)
    assert (got1 == orc.to_ref160(w1)).all()
    assert (got2 == orc.to_ref160(w2)).all()
    # the other formats, each twice (the mark stays valid across exports)
    for _ in range(2):
        assert (c1.to_bytes_folded() == orc.encode(w1, 8)).all()
        assert (c2.to_packed().reshape(n, -1) == np.asarray(w2).view(np.uint8).reshape(n, -1)).all()
        assert (c1.to_bytes_affine() == orc.to_affine(w1)).all()
    # an ordered export (after a read of c1 by another call) gives the same bytes
    c1.equal(c1)
    assert (raw(ft, c1) == got1).all()


def test_write_after_mark_is_seen(ft, orc):
    """c *= k marks c; c += d afterwards is an unmarked write: the export
    must wait for it (ordered path) and show the sum."""
    g = synth.rng(72)
    n = 5000
    p = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    d = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    k = synth.scalars_mod_L(g, n)
    want = orc.encode(orc.add(orc.mul(p, k, threads=8), d, threads=8), 8)
    c, dd = ft.Array.from_packed(p), ft.Array.from_packed(d)
    c.mul(k)
    c.add(dd)
    assert (c.to_bytes_folded() == want).all()
    # a later mark makes the overlapped path valid again
    k2 = synth.scalars_mod_L(g, n)
    c.mul(k2)
    want2 = orc.encode(orc.mul(orc.add(orc.mul(p, k, threads=8), d, threads=8), k2, threads=8), 8)
    assert (c.to_bytes_folded() == want2).all()


def test_batch_write_after_mark_is_seen(ft, orc):
    """A batch run writes arrays through recorded addresses: an export after
    it shows the batch's result, not the marked state before it."""
    g = synth.rng(73)
    n = 3000
    p = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    d = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    k = synth.scalars_mod_L(g, n)
    c, dd = ft.Array.from_packed(p), ft.Array.from_packed(d)
    b = ft.Batch()
    b.add(c, dd)
    c.mul(k)  # marks c after the batch was recorded
    b.run()
    want = orc.encode(orc.add(orc.mul(p, k, threads=8), d, threads=8), 8)
    assert (c.to_bytes_folded() == want).all()
    b.free()


def test_write_through_device_view_is_seen(ft, orc):
    """After ftx_array_device_view the caller may write the storage itself
    (here: ftx_scan_noalloc on the library stream): exports of that array
    stay in stream order and show the write."""
    g = synth.rng(74)
    n = 4096
    p = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    k = synth.scalars_mod_L(g, n)
    c = ft.Array.from_packed(p)
    c.mul(k)
    planes, stride = c.device_view()
    L = ft.api.lib()
    ft.check(L.ftx_scan_noalloc(ctypes.c_void_p(planes), stride, n, 0, ctypes.c_void_p(ft.stream_handle())))
    want = orc.encode(orc.scan(orc.mul(p, k, threads=8), False, threads=8), 8)
    assert (c.to_bytes_folded() == want).all()
    c.mul(k)  # marks after the view was handed out: still ordered
    assert (c.to_bytes_folded() == orc.encode(orc.mul(orc.scan(orc.mul(p, k, threads=8), False, threads=8), k,
                                                      threads=8), 8)).all()


def test_pinned_scalar_staging_ring(ft, orc):
    """ft_mul with pinned scalars alternates two staging buffers, grows them
    when a larger call comes, and may reuse a buffer while an earlier ladder
    still reads the other one: every product equals the oracle's."""
    torch = pytest.importorskip("torch")
    g = synth.rng(75)
    sizes = [100, 20000, 7, 20000, 65537, 3]
    arrs, wants = [], []
    for n in sizes:
        p = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
        k1 = synth.scalars_mod_L(g, n)
        k2 = synth.scalars_mod_L(g, n)
        a = ft.Array.from_packed(p)
        a.mul(pinned(torch, k1))
        a.mul(k2)  # pageable: the ordered path in between
        a.mul(pinned(torch, k1))
        arrs.append(a)
        wants.append(orc.mul(orc.mul(orc.mul(p, k1, threads=8), k2, threads=8), k1, threads=8))
    for a, w in zip(arrs, wants):
        assert (a.to_bytes_folded() == orc.encode(w, 8)).all()


def test_server_write_after_mark_is_seen(ft, orc):
    """c1, c2 marked by ft_mul, then multiplied in place by a server request
    (on the server's own stream): once the request's result is taken, the
    exports show the server's product, not the marked state."""
    g = synth.rng(76)
    n = 2500
    p1 = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    p2 = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    k1 = synth.scalars_mod_L(g, n)
    k2 = synth.scalars_mod_L(g, n)
    c1, c2 = ft.Array.from_packed(p1), ft.Array.from_packed(p2)
    c1.mul(k1)
    c2.mul(k1)
    sk = synth.scalars_mod_L(g, 1)
    pk = ft.Array.from_scalars(sk).to_bytes_folded()[0]
    srv = ft.Server(pk, 1 << 30, slots=2)
    try:
        t = srv.submit_smul(c1, c2, k2)
        srv.wait(t)
        assert (c1.to_bytes_folded() == orc.encode(orc.mul(orc.mul(p1, k1, threads=8), k2, threads=8), 8)).all()
        assert (c2.to_bytes_folded() == orc.encode(orc.mul(orc.mul(p2, k1, threads=8), k2, threads=8), 8)).all()
    finally:
        srv.close()


def test_length_changes_after_mark(ft, orc):
    """A marked array shortened in place (to more than half its length: same
    storage) exports its first n points on the overlapped path; lengthened
    (the new points set to the identity, a use of the storage) or shortened
    to half or less (new storage) it exports in stream order."""
    torch = pytest.importorskip("torch")
    g = synth.rng(77)
    n = 3001
    p = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
    k = synth.scalars_mod_L(g, n)
    want = orc.encode(orc.mul(p, k, threads=8), 8)
    ident = ft.Array.init_scalar(1).to_bytes_folded()[0]
    c = ft.Array.from_packed(p)
    c.mul(pinned(torch, k))
    c.set_length(2000)
    assert (c.to_bytes_folded() == want[:2000]).all()
    c.set_length(2600)
    got = c.to_bytes_folded()
    assert (got[:2000] == want[:2000]).all() and (got[2000:] == ident).all()
    c.set_length(6000)
    got = c.to_bytes_folded()
    assert (got[:2000] == want[:2000]).all() and (got[2000:] == ident).all()
    c.mul(pinned(torch, np.tile(k[:1], (6000, 1))))
    c.set_length(1000)
    assert (c.to_bytes_folded() == orc.encode(orc.mul(orc.mul(p[:1000], k[:1000], threads=8),
                                                      np.tile(k[:1], (1000, 1)), threads=8), 8)).all()
    # one point, pinned scalars, export right away
    one = ft.Array.from_packed(p[:1])
    one.mul(pinned(torch, k[:1]))
    assert (raw(ft, one, torch) == orc.to_ref160(orc.mul(p[:1], k[:1]))).all()


@pytest.mark.parametrize("n", [291840, 300001])
def test_mul_in_two_parts_then_exports(ft, orc, n):
    """ft_mul over four or more waves of the ladder launch runs as two
    launches (every whole wave but the last, then the rest), marked as two
    parts, and its exports copy the first part while the second computes.
    291,840 points are five whole waves at 152 SMs x 384 threads (the cut on
    a wave boundary, a full last part), 300,001 cut inside the last wave.
    Every format equals the oracle, with a second multiplication queued
    behind, for pinned and pageable scalars, and after the length shrank
    (past the cut: a shorter second part; below it: the export waits for
    the whole call)."""
    torch = pytest.importorskip("torch")
    g = synth.rng(80 + n % 7)
    p = ft.Array.from_scalars(synth.scalars_mod_L(g, n)).to_packed()
    k = synth.scalars_mod_L(g, n)
    w = orc.mul(p, k, threads=16)
    c, c2 = ft.Array.from_packed(p), ft.Array.from_packed(p)
    hk = pinned(torch, k)
    c.mul(hk)
    c2.mul(hk)
    assert (raw(ft, c, torch) == orc.to_ref160(w)).all()
    assert (c.to_bytes_folded() == orc.encode(w, 16)).all()
    assert (c.to_bytes_affine() == orc.to_affine(w)).all()
    assert (c.to_packed() == w).all()
    assert (c2.to_packed() == w).all()
    c3 = ft.Array.from_packed(p)
    c3.mul(k)
    assert (raw(ft, c3) == orc.to_ref160(w)).all()
    # shorter, without a reallocation (above half the length): still past
    # the cut, then below it
    for m in (n - 5000, int(n * 0.6)):
        c4 = ft.Array.from_packed(p)
        c4.mul(hk)
        c4.set_length(m)
        assert (c4.to_bytes_folded() == orc.encode(w[:m], 16)).all()
