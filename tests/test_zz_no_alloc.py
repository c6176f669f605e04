"""ftx_scan_noalloc, the allocation-free scan for callers that cannot call
cudaMalloc (their device memory is held by another allocator, or they must
avoid cudaMalloc's synchronisation): called through the C ABI on the
caller's own device buffer and stream, its result must equal ft_array_scan /
ft_array_prescan on the same points, byte for byte, on two calls in a row
(the second call finds the first call's partial sums still in the shared
scratch array).  Collected last so a run stopping at the first failure has
already run every other test; passes alone in a fresh process too."""
import ctypes

import numpy as np
import pytest

from libftcrypto_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_POINTS = 1048576  # FT_NOALLOC_SCAN_MAX_POINTS in include/ftcrypto_gb300.h


def noalloc_scan(ft, arr, exclusive, stream=None):
    """One call through the C ABI on `stream` (a stream the caller owns), or
    on the library's stream; returns after the scan has finished."""
    L = ft.api.lib()
    planes, stride = arr.device_view()
    ft.synchronize()  # the array's producer ran on the library's stream
    code = L.ftx_scan_noalloc(ctypes.c_void_p(planes), stride, len(arr), exclusive,
                              ctypes.c_void_p(stream.cuda_stream if stream is not None else ft.stream_handle()))
    ft.check(code)
    if stream is not None:
        stream.synchronize()
    ft.synchronize()


@pytest.mark.parametrize("exclusive", [0, 1])
def test_noalloc_scan_matches_ft_array_scan_twice(ft, orc, exclusive):
    g = synth.rng(900 + exclusive)
    for n in (70001, 3000):  # two calls in a row, the second smaller
        pts = orc.from_scalars(synth.scalars_mod_L(g, n), threads=8)
        mine = ft.Array.from_packed(pts)
        noalloc_scan(ft, mine, exclusive)
        ref = ft.Array.from_packed(pts)
        if exclusive:
            ref.prescan()
        else:
            ref.scan()
        assert (mine.to_bytes_folded() == ref.to_bytes_folded()).all()


def test_noalloc_scan_largest_and_too_large(ft, orc):
    g = synth.rng(902)
    base = ft.Array.from_scalars(synth.scalars_mod_L(g, 1024))
    big = ft.Array.init_point(MAX_POINTS, base, 7)
    big.add(ft.Array.init_point(MAX_POINTS, base, 3))
    ref = big.get_range(0, MAX_POINTS, 1)
    noalloc_scan(ft, big, 0)
    ref.scan()
    idx = np.sort(g.choice(MAX_POINTS, 256, replace=False))
    assert (big.get_subset(idx).to_bytes_folded() == ref.get_subset(idx).to_bytes_folded()).all()
    # one point more than the stated maximum is refused before any launch
    L = ft.api.lib()
    planes, stride = big.device_view()
    code = L.ftx_scan_noalloc(ctypes.c_void_p(planes), MAX_POINTS + 1, MAX_POINTS + 1, 0,
                              ctypes.c_void_p(ft.stream_handle()))
    assert code == 3  # FT_ERR_BAD_SIZE


def test_noalloc_scan_on_callers_stream_allocates_nothing(ft, orc):
    """The use the entry point exists for: the caller's own stream, and no
    device memory taken by the call (the device's free memory, which any
    cudaMalloc or growth of the library's pool would lower, is unchanged)."""
    torch = pytest.importorskip("torch")
    g = synth.rng(903)
    n = 200_003
    pts = orc.from_scalars(synth.scalars_mod_L(g, 4096), threads=8)
    pts = np.tile(pts, (n // 4096 + 1, 1))[:n].copy()
    ref = ft.Array.from_packed(pts)
    ref.scan()
    want = ref.to_bytes_folded()
    st = torch.cuda.Stream()
    for _ in range(2):  # the second call finds the first call's partial sums in the array
        mine = ft.Array.from_packed(pts)
        noalloc_scan(ft, mine, 0, st)  # first call on this device: the address lookup
        free0, _ = ft.device_memory()
        mine2 = ft.Array.from_packed(pts)
        ft.synchronize()
        free1, _ = ft.device_memory()
        noalloc_scan(ft, mine2, 0, st)
        free2, _ = ft.device_memory()
        assert free2 == free1, "the call took device memory"
        assert free1 <= free0
        assert (mine.to_bytes_folded() == want).all()
        assert (mine2.to_bytes_folded() == want).all()
