"""The batch autotuner's persistent cache (host side, no GPU)."""

import json

from awkward_gb300 import batch


def test_cache_roundtrip(tmp_path):
    path = str(tmp_path / "sub" / "tune.json")
    k1 = batch.cache_key(((10, 3, 5),), "GPU X", "v1")
    k2 = batch.cache_key(((11, 2, 7),), "GPU X", "v1")
    batch._cache_store(path, k1, batch.PlanKnobs(0, 2, 1024, 128))
    batch._cache_store(path, k2, batch.PlanKnobs())
    d = batch._cache_load(path)
    assert batch.PlanKnobs(**d[k1]) == batch.PlanKnobs(0, 2, 1024, 128)
    assert batch.PlanKnobs(**d[k2]) == batch.PlanKnobs()
    assert json.load(open(path)) == d


def test_cache_tolerates_a_broken_file(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    assert batch._cache_load(str(path)) == {}
    assert batch._cache_load(str(tmp_path / "missing.json")) == {}


def test_waves_keep_order_and_respect_the_size_limit():
    specs = batch.batch_specs(300, seed=5, min_lists=1_000, max_lists=2_000_000)
    ws = batch.waves(specs, 8e9)
    assert [s for w in ws for s in w] == specs
    for w in ws:
        assert len(w) == 1 or sum(batch.spec_bytes(s) for s in w) <= 8e9
    # the same array gets the same seed whatever the wave split
    assert [s[3] for s in specs] == [5 * 1_000_003 + a for a in range(300)]
