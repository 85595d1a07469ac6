"""Autotuner cache logic (no GPU): classes, flag bits, persistence."""
import json

from fast_matched_filter_gb300 import _lib, autotune


def test_cache_roundtrip_and_flags(tmp_path, monkeypatch):
    monkeypatch.setenv("FMF_AUTOTUNE_CACHE", str(tmp_path / "tiles.json"))
    assert autotune.lookup(600, 1, 60, "short", "split_bf16") is None
    assert autotune.flags_for(600, 1, 60, "short", "split_bf16") == 0
    table = {autotune.search_class(600, 1, 60, "short", "split_bf16"):
             {"lag_blocks": 64, "template_group": 8}}
    autotune._save(table)
    assert json.loads((tmp_path / "tiles.json").read_text()) == table
    assert autotune.lookup(600, 1, 60, "short", "split_bf16") == (64, 8)
    f = autotune.flags_for(600, 1, 60, "short", "split_bf16")
    assert f == _lib.flag_tile(64) | _lib.flag_template_group(8)
    assert (f >> 8) & 0xFF == 4 and (f >> 16) & 0xFF == 8
    # the plain form has no tile shape; other classes are independent
    assert autotune.flags_for(600, 1, 60, "short", "fp32") == 0
    assert autotune.lookup(600, 2, 60, "short", "split_bf16") is None
