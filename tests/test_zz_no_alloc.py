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


def noalloc_scan(ft, arr, exclusive):
    L = ft.api.lib()
    planes, stride = arr.device_view()
    code = L.ftx_scan_noalloc(ctypes.c_void_p(planes), stride, len(arr), exclusive,
                              ctypes.c_void_p(ft.stream_handle()))
    ft.check(code)
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
