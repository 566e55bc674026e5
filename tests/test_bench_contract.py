"""The reference arm of bench.py on the CPU: one JSON line with the contract's keys.

The GPU arm needs a GPU; the reference arm times the oracle port of awkward-cpp's CPU
reducers on the host cores, so its line (and the torchrun behaviour: rank 0 alone prints)
can be checked here on a small list count.
"""

import json
import os
import socket
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--lists", "50000"], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["lists_per_gpu"] == 50000 and "workload" in d["config"]
    # the GPU arm builds its config with the same function (same keys, same workload)
    sys.path.insert(0, ROOT)
    import bench

    assert d["config"] == bench.c1_config(50000, d["config"]["elements_per_gpu"], 1)
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_on_rank_zero_only():
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(_free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1", "--lists", "20000"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def test_bench_shards_concatenate_to_one_global_array():
    sys.path.insert(0, ROOT)
    import numpy as np

    import bench

    world = 3
    parts = [bench.make_c1_shard(5000, r, world) for r in range(world)]
    glob = np.concatenate([parts[0][2]] + [p[2][1:] for p in parts[1:]])
    assert glob[0] == 0 and len(glob) == world * 5000 + 1
    for r, (local, x, gslice, l0) in enumerate(parts):
        np.testing.assert_array_equal(local, gslice - gslice[0])
        assert len(x) == local[-1] and (r == 0 or l0 > 0)
    off1, x1, g1, l01 = bench.make_c1_shard(5000, 0, 1)
    off0, x0 = bench.make_c1(5000, 0)
    np.testing.assert_array_equal(off1, off0) and np.testing.assert_array_equal(x1, x0)
    assert l01 == 0
