"""Launch-shape tuner, host side: candidates, size classes and the JSON cache
(no GPU needed; the library only answers its compiled block bounds)."""

import json

from opensss_gb300 import autotune


def test_pair_warp_candidates_stay_within_the_compiled_bound():
    assert autotune.pair_warp_candidates(13) == [4, 8, 12]
    assert autotune.pair_warp_candidates(16) == [4, 8, 12]
    assert autotune.pair_warp_candidates(33) == [4, 8]
    assert autotune.pair_warp_candidates(13, kahan=True) == [4, 8]
    assert autotune.pair_warp_candidates(1) == [4, 8, 12]


def test_size_classes_round_up_to_powers_of_two():
    a = autotune.size_class("GB300", 13, 768, (64, 64, 48))
    b = autotune.size_class("GB300", 13, 700, (60, 64, 48))
    c = autotune.size_class("GB300", 33, 768, (64, 64, 48))
    assert a == b and a != c
    assert "kahan=1" in autotune.size_class("GB300", 13, 768, (64, 64, 48), kahan=True)


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "shapes.json"
    monkeypatch.setenv("OPENSSS_GB300_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_memory", {})
    key = autotune.size_class("dev", 13, 768, (64, 64, 48))
    assert autotune.lookup(key) is None
    autotune._store(key, {"pair_warps": 8, "leg_threads": 64})
    assert json.loads(path.read_text())[key]["pair_warps"] == 8
    assert autotune.lookup(key) == {"pair_warps": 8, "leg_threads": 64}
    path.write_text("not json")  # a damaged cache reads as empty
    monkeypatch.setattr(autotune, "_memory", {})
    assert autotune.lookup(key) is None
