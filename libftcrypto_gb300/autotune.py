"""Autotuner for the library's run-time launch-shape knobs (ftx_tune).

Knobs and candidates:
  FTX_TUNE_LADDER_BLOCK   block size of the variable-base ladder: 128, 192,
                          224 threads with the 1 KB per-thread tables in
                          shared memory, or 384, 448 with half of each table
                          in tensor memory (this sets how many warps an SM
                          holds, against registers per thread)
  FTX_TUNE_BATCH_ADD_PTS  points per thread of an ADD item of the batched
                          form: 1, 2, 4, 8, 16 (item granularity against
                          queue overhead)
  FTX_TUNE_SCALE_WINDOW   window width of the small-scalar ladder
                          (ftx_scale_bounded, batched scales): 2, 3, 4 bits,
                          timed on an uneven batch of scales by k below 2^10,
                          the bound of the batched workload (table of 2, 4 or
                          8 entries against the number of windows; the points
                          are the same).  Timed in the batched kernel, where
                          the setting matters: on one long array widths 2 and
                          3 time alike, in the batched mix 3 is 9-15% faster.
The window width of the 253-bit variable-base ladder is not a knob: the
reference's 4-bit signed window is kept there (it is also the minimum of
field operations for 253-bit scalars, and an 8-entry table per thread is
what the SM's shared and tensor memory hold).

Each candidate is timed on the device (best of five, synchronised wall
clock) and the fastest is applied.  Results are cached per GPU model in
$FT_TUNE_CACHE (default ~/.cache/libftcrypto_gb300/tune.json).
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import api, synth

CANDIDATES = {
    api.TUNE_LADDER_BLOCK: (128, 192, 224, 384, 448),
    api.TUNE_BATCH_ADD_PTS: (1, 2, 4, 8, 16),
    api.TUNE_SCALE_WINDOW: (2, 3, 4),
}
NAMES = {api.TUNE_LADDER_BLOCK: "ladder_block", api.TUNE_BATCH_ADD_PTS: "batch_add_pts",
         api.TUNE_SCALE_WINDOW: "scale_window"}
SCALE_BITS = 10  # the bound of the batched workload's scalars (k <= 1000)


def cache_path() -> str:
    return os.environ.get("FT_TUNE_CACHE", os.path.expanduser("~/.cache/libftcrypto_gb300/tune.json"))


def _best_of(fn, reps=5):
    best = float("inf")
    for _ in range(reps):
        api.synchronize()
        t = time.perf_counter()
        fn()
        api.synchronize()
        best = min(best, time.perf_counter() - t)
    return best


def device_key() -> str:
    free, total = api.device_memory()
    return f"sm103-{total >> 30}GiB"


def tune(n_points: int = 1 << 18, seed: int = 7) -> dict:
    """Time every candidate and apply the fastest; returns {knob: value}."""
    g = synth.rng(seed)
    sc = synth.scalars_mod_L(g, n_points)
    base = api.Array.from_scalars(sc)
    work = base.get_range(0, n_points, 1)
    timings = {}
    best = {}
    for v in CANDIDATES[api.TUNE_LADDER_BLOCK]:
        api.tune(api.TUNE_LADDER_BLOCK, v)
        timings[f"ladder_block={v}"] = _best_of(lambda: work.mul(sc))
    best[api.TUNE_LADDER_BLOCK] = min(CANDIDATES[api.TUNE_LADDER_BLOCK],
                                      key=lambda v: timings[f"ladder_block={v}"])
    api.tune(api.TUNE_LADDER_BLOCK, best[api.TUNE_LADDER_BLOCK])
    # an uneven add-only batch: lengths log-uniform in [1, 65536]
    lens = np.clip(np.floor(np.exp(g.uniform(0, np.log(65536), 256))), 1, 65536).astype(int)
    pairs = [(base.get_range(0, min(n, n_points), 1), base.get_range(0, min(n, n_points), 1)) for n in lens]
    for v in CANDIDATES[api.TUNE_BATCH_ADD_PTS]:
        api.tune(api.TUNE_BATCH_ADD_PTS, v)
        b = api.Batch()
        for x, y in pairs:
            b.add(x, y)
        b.run()
        timings[f"batch_add_pts={v}"] = _best_of(b.run)
        b.free()
    best[api.TUNE_BATCH_ADD_PTS] = min(CANDIDATES[api.TUNE_BATCH_ADD_PTS],
                                       key=lambda v: timings[f"batch_add_pts={v}"])
    api.tune(api.TUNE_BATCH_ADD_PTS, best[api.TUNE_BATCH_ADD_PTS])
    # small-scalar ladder width at the batched workload's bound, on an
    # uneven batch of scales (the width is fixed when a batch is uploaded)
    scale_arrs = [x for x, _ in pairs]
    for v in CANDIDATES[api.TUNE_SCALE_WINDOW]:
        api.tune(api.TUNE_SCALE_WINDOW, v)
        b = api.Batch()
        for x in scale_arrs:
            b.scale_small(x, 1000, SCALE_BITS)
        b.run()
        timings[f"scale_window={v}"] = _best_of(b.run)
        b.free()
    best[api.TUNE_SCALE_WINDOW] = min(CANDIDATES[api.TUNE_SCALE_WINDOW],
                                      key=lambda v: timings[f"scale_window={v}"])
    api.tune(api.TUNE_SCALE_WINDOW, best[api.TUNE_SCALE_WINDOW])
    result = {NAMES[k]: v for k, v in best.items()}
    result["timings_s"] = timings
    return result


def load_or_tune(force: bool = False) -> dict:
    """Apply the cached choice for this GPU model, tuning first if needed."""
    path = cache_path()
    key = device_key()
    cache = {}
    if os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if force or key not in cache or any(name not in cache[key] for name in NAMES.values()):
        cache[key] = tune()
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    entry = cache[key]
    for knob, name in NAMES.items():
        if name in entry:
            api.tune(knob, entry[name])
    return entry
