"""The autotuner applies a supported value for every knob and caches it."""
import json

import pytest

pytestmark = pytest.mark.gpu


def test_autotune_applies_and_caches(ft, tmp_path, monkeypatch):
    from libftcrypto_gb300 import autotune
    monkeypatch.setenv("FT_TUNE_CACHE", str(tmp_path / "tune.json"))
    entry = autotune.load_or_tune(force=True)
    assert entry["ladder_block"] in (128, 192, 224, 384, 448)
    assert ft.tune_get(ft.TUNE_LADDER_BLOCK) == entry["ladder_block"]
    assert ft.tune_get(ft.TUNE_BATCH_ADD_PTS) == entry["batch_add_pts"]
    assert entry["scale_window"] in (2, 3, 4)
    assert ft.tune_get(ft.TUNE_SCALE_WINDOW) == entry["scale_window"]
    cached = json.load(open(tmp_path / "tune.json"))
    assert list(cached.values())[0]["ladder_block"] == entry["ladder_block"]
    with pytest.raises(ft.FtError):
        ft.tune(ft.TUNE_LADDER_BLOCK, 100)
