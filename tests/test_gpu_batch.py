"""GPU tests of the batched path: one launch per operation over many arrays.

Every plan variant the autotuner can choose, replayed from a CUDA graph,
must give outputs bit-identical to the per-array entry points (sum, max,
argmax, count and array[mask]) on a batch of uneven arrays: Poisson and
geometric (heavy-tailed) lengths, empty lists, an array without lists, an
array of only empty lists and one holding a 300,000-element list (giant-list
records across warp ranges).
"""

import math

import numpy as np
import pytest
import torch  # noqa: F401  (CUDA context for the generators below)

pytestmark = pytest.mark.gpu


def _special_arrays():
    import torch

    dev = "cuda"
    gen = torch.Generator(device=dev).manual_seed(99)
    out = []
    for L in (torch.tensor([], dtype=torch.int64), torch.zeros(1000, dtype=torch.int64),
              torch.tensor([3, 0, 300_000, 5, 0, 7], dtype=torch.int64)):
        L = L.to(dev)
        off = torch.zeros(L.numel() + 1, dtype=torch.int64, device=dev)
        if L.numel():
            torch.cumsum(L, 0, out=off[1:])
        E = int(off[-1].item())
        x = torch.randn(E, dtype=torch.float64, device=dev, generator=gen)
        m = torch.rand(E, device=dev, generator=gen) < 0.4
        out.append((off, x, m))
    return out


def _batch():
    from awkward_gb300 import batch

    b = batch.make_batch(48, seed=3, min_lists=100, max_lists=30_000)
    return batch.Batch(b.arrays[:20] + _special_arrays() + b.arrays[20:])


def _variants():
    from awkward_gb300 import batch

    return batch.PLAN_VARIANTS


@pytest.mark.parametrize("variant", _variants(), ids=lambda k: f"o{k.order_mode}d{k.occupancy_div}r{k.range_min}b{k.block}")
def test_batched_graph_matches_per_array(variant):
    import torch

    from awkward_gb300 import batch

    b = _batch()
    plan = b.plan(variant)
    g = b.graph(plan)
    for _ in range(2):  # replays recompute everything from scratch
        g.replay()
    torch.cuda.synchronize()
    b.check_errors()
    got = b.outputs()
    exp = batch.run_plain(b)
    for i, (gi, ei) in enumerate(zip(got, exp)):
        for name, x, y in zip(("sum", "max", "argmax", "count", "sel_offsets", "sel_content"), gi, ei):
            assert x.shape == y.shape, (i, name)
            if x.dtype == torch.float64:
                assert torch.equal(x.view(torch.int64), y.view(torch.int64)), (i, name)
            else:
                assert torch.equal(x, y), (i, name)
    b.close()


def test_autotune_caches_by_shape(tmp_path, monkeypatch):
    import json

    from awkward_gb300 import batch

    monkeypatch.setenv(batch.CACHE_ENV, str(tmp_path / "tune.json"))
    batch._TUNED.clear()
    b = batch.make_batch(16, seed=4, min_lists=100, max_lists=5_000)
    v = batch.autotune(b, reps=1)
    assert isinstance(v, batch.PlanKnobs)
    for name, values in batch.KNOB_VALUES.items():
        assert getattr(v, name) in values
    stored = json.load(open(tmp_path / "tune.json"))
    assert len(stored) == 1 and list(stored.values())[0] == {
        "order_mode": v.order_mode, "occupancy_div": v.occupancy_div,
        "range_min": v.range_min, "block": v.block}
    assert batch.autotune(b) == v
    batch._TUNED.clear()  # a new process: the file answers without timing
    assert batch.autotune(b) == v
    b.close()
    assert math.isfinite(batch.time_plain(b))
