"""Batched jagged operations: many arrays, one launch per operation, one CUDA graph.

``Batch`` holds A float64 ListOffsetArrays ``(offsets, content)`` with one
jagged boolean mask each (CUDA tensors) and the outputs of

    sum, max, argmax, count (axis=-1)   and   array[mask]

for every array.  ``Batch.plan(knobs)`` builds the device
work queue (libawkward_gb300's batch plan); ``Batch.graph(plan)`` captures one
run of every operation in a CUDA graph, and ``graph.replay()`` re-runs it.

``autotune(batch)`` picks the plan's knobs -- dequeue order, persistent CTAs
per SM, the range size of arrays whose lists are all short, threads per
reducer CTA -- by timing graph replays on the batch itself (coordinate
descent from the default, one knob at a time), keyed by a signature of the
batch's length histogram (arrays per power-of-two bucket of list count and
of mean list length), the device and the library version.  Winners are kept
in the process and in a JSON file (``AWKWARD_GB300_TUNE_CACHE``, default
``~/.cache/awkward_gb300/batch_tune.json``), so later processes reuse them.

``make_wave(specs, ...)`` generates a subset of a batch distribution on the
device from per-array seeds, so a distribution too large for device memory
is run as a sequence of resident waves whose union is the same batch
whatever the wave split.

``run_plain(batch)`` runs the same operations array by array through the
per-array entry points (awkward's own sequence of calls, with its host
reads of data-dependent sizes) -- the reference the batched outputs equal
bit for bit.
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import time
from dataclasses import asdict, dataclass

import numpy as np
import torch

from . import _abi
from .kernel_table import backend


@dataclass(frozen=True)
class PlanKnobs:
    """The tuning knobs of a batch plan (awkward_gb300_batch_plan_create)."""

    order_mode: int = 1      # 0: items in array order; 1: largest ranges first
    occupancy_div: int = 1   # persistent CTAs per SM = occupancy / occupancy_div
    range_min: int = 4096    # items per range of arrays with only short lists
    block: int = 256         # threads per reducer CTA


KNOB_VALUES = {"order_mode": (0, 1), "occupancy_div": (1, 2),
               "range_min": (1024, 4096, 16384), "block": (128, 256)}
# the variants every test replays (bit-identical outputs whatever the knobs)
PLAN_VARIANTS = [PlanKnobs(0, 1), PlanKnobs(1, 1), PlanKnobs(1, 2), PlanKnobs(0, 2),
                 PlanKnobs(1, 1, 1024, 128), PlanKnobs(0, 1, 16384, 256)]
_TUNED = {}
CACHE_ENV = "AWKWARD_GB300_TUNE_CACHE"


def cache_path():
    return os.environ.get(CACHE_ENV) or os.path.join(
        os.path.expanduser("~"), ".cache", "awkward_gb300", "batch_tune.json")


def _cache_load(path):
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _cache_store(path, key, knobs):
    """Add one winner to the JSON cache (read-modify-write, atomic replace)."""
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        d = _cache_load(path)
        d[key] = asdict(knobs)
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # an unwritable cache only costs a re-tune in the next process


def cache_key(signature, device_name, version):
    return f"{device_name}|{version}|{json.dumps(signature)}"


class Batch:
    def __init__(self, arrays):
        """arrays: list of (offsets int64 [n+1], content float64 [E], mask bool [E])."""
        self.arrays = arrays
        dev = arrays[0][0].device
        self.device = dev
        ends = torch.stack([torch.stack([o[0], o[-1]]) for o, _c, _m in arrays]).cpu().numpy()
        self.nlists = np.array([o.numel() - 1 for o, _c, _m in arrays], np.int64)
        self.nelements = (ends[:, 1] - ends[:, 0]).astype(np.int64)
        # longest list of each array (decides whether its reduction ranges may be widened)
        self.maxlen = torch.stack([
            (o[1:] - o[:-1]).max() if o.numel() > 1 else torch.zeros((), dtype=o.dtype, device=o.device)
            for o, _c, _m in arrays]).cpu().numpy().astype(np.int64)
        self.out_sum, self.out_max, self.out_argmax, self.out_count = [], [], [], []
        self.sel_offsets, self.sel_content = [], []
        for (o, c, m), n in zip(arrays, self.nlists):
            self.out_sum.append(torch.empty(max(n, 1), dtype=torch.float64, device=dev))
            self.out_max.append(torch.empty(max(n, 1), dtype=torch.float64, device=dev))
            self.out_argmax.append(torch.empty(max(n, 1), dtype=torch.int64, device=dev))
            self.out_count.append(torch.empty(max(n, 1), dtype=torch.int64, device=dev))
            # zeroed: an array without lists has no select tile to write its offsets[0]
            self.sel_offsets.append(torch.zeros(n + 1, dtype=torch.int64, device=dev))
            self.sel_content.append(torch.empty(max(c.numel(), 1), dtype=torch.float64, device=dev))
        self.err = torch.full((1,), -1, dtype=torch.int64, device=dev)
        self._plans = []

    def signature(self):
        """Histogram of the batch's shape: arrays per (log2 list count, log2 mean length)."""
        mean = self.nelements / np.maximum(self.nlists, 1)
        a = np.floor(np.log2(np.maximum(self.nlists, 1))).astype(int)
        b = np.floor(np.log2(np.maximum(mean, 1))).astype(int)
        keys, counts = np.unique(np.stack([a, b], 1), axis=0, return_counts=True)
        return tuple((int(k[0]), int(k[1]), int(c)) for k, c in zip(keys, counts))

    def _ptrs(self, tensors):
        return np.array([t.data_ptr() for t in tensors], np.uint64)

    def plan(self, knobs=None, occupancy_div=None):
        """A device plan with the given PlanKnobs (or (order_mode, occupancy_div))."""
        if not isinstance(knobs, PlanKnobs):
            knobs = PlanKnobs(1 if knobs is None else int(knobs),
                              1 if occupancy_div is None else int(occupancy_div))
        tables = [self.nlists, self.nelements, self.maxlen,
                  self._ptrs([c for _o, c, _m in self.arrays]),
                  self._ptrs([o for o, _c, _m in self.arrays]),
                  self._ptrs([m for _o, _c, m in self.arrays]),
                  self._ptrs(self.out_sum), self._ptrs(self.out_max), self._ptrs(self.out_argmax),
                  self._ptrs(self.out_count), self._ptrs(self.sel_offsets),
                  self._ptrs(self.sel_content)]
        handle = ctypes.c_void_p()
        rc = _abi.ext_cfunc("awkward_gb300_batch_plan_create")(
            ctypes.addressof(handle), len(self.arrays), *[t.ctypes.data for t in tables],
            knobs.order_mode, knobs.occupancy_div, knobs.range_min, knobs.block,
            self.err.data_ptr())
        if rc != 0:
            raise RuntimeError(f"awkward_gb300_batch_plan_create: cudaError {rc}")
        self._plans.append(handle)
        return handle

    def run(self, plan):
        rc = _abi.ext_cfunc("awkward_gb300_batch_plan_run")(
            plan, torch.cuda.current_stream(self.device).cuda_stream)
        if rc != 0:
            raise RuntimeError(f"awkward_gb300_batch_plan_run: cudaError {rc}")

    def graph(self, plan):
        """A CUDA graph of one run of the plan (warmed up once outside capture)."""
        self.run(plan)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(plan)
        return g

    def check_errors(self):
        word = int(self.err.item()) & ((1 << 64) - 1)
        if word != (1 << 64) - 1:
            raise ValueError("GPU kernel gave up waiting for a predecessor tile "
                             "(bounded wait exceeded) in compiled CUDA code (batch select)")

    def outputs(self):
        """Per array: (sum, max, argmax, count, sel_offsets, sel_content) trimmed to size."""
        out = []
        for i, n in enumerate(self.nlists):
            so = self.sel_offsets[i]
            k = int(so[-1].item()) if n > 0 else 0
            out.append((self.out_sum[i][:n], self.out_max[i][:n], self.out_argmax[i][:n],
                        self.out_count[i][:n], so, self.sel_content[i][:k]))
        return out

    def close(self):
        for h in self._plans:
            _abi.ext_cfunc("awkward_gb300_batch_plan_destroy")(h)
        self._plans = []


def time_plan(batch, knobs, reps=3):
    """Mean replay time (ms) of a CUDA graph of the plan with `knobs`."""
    plan = batch.plan(knobs)
    g = batch.graph(plan)
    g.replay()
    torch.cuda.synchronize(batch.device)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        g.replay()
    b.record()
    torch.cuda.synchronize(batch.device)
    del g
    return a.elapsed_time(b) / reps


def autotune(batch, reps=3, persist=True):
    """The PlanKnobs of the fastest plan for this batch's shape.

    Coordinate descent from PlanKnobs(): each knob in turn is set to each of
    its values (the others fixed at the best so far) and the graph replay
    timed on the batch.  Results are cached per (device, library version,
    length-histogram signature) in the process and, with `persist`, in the
    JSON file at cache_path().
    """
    sig = batch.signature()
    dev_name = torch.cuda.get_device_name(batch.device)
    key = cache_key(sig, dev_name, _abi.version())
    if key in _TUNED:
        return _TUNED[key]
    if persist:
        hit = _cache_load(cache_path()).get(key)
        if isinstance(hit, dict):
            try:
                knobs = PlanKnobs(**hit)
                _TUNED[key] = knobs
                return knobs
            except TypeError:
                pass
    best = PlanKnobs()
    best_ms = time_plan(batch, best, reps)
    for name, values in KNOB_VALUES.items():
        for v in values:
            cand = PlanKnobs(**{**asdict(best), name: v})
            if cand == best:
                continue
            ms = time_plan(batch, cand, reps)
            if ms < best_ms:
                best, best_ms = cand, ms
    _TUNED[key] = best
    if persist:
        _cache_store(cache_path(), key, best)
    return best


def run_plain(batch):
    """The same operations through the per-array entry points, array by array."""
    from . import jagged

    be = backend()
    outs = []
    for (o, c, m), n in zip(batch.arrays, batch.nlists):
        s = torch.empty(n, dtype=torch.float64, device=batch.device)
        mx = torch.empty(n, dtype=torch.float64, device=batch.device)
        am = torch.empty(n, dtype=torch.int64, device=batch.device)
        ct = torch.empty(n, dtype=torch.int64, device=batch.device)
        if n > 0:
            be["awkward_reduce_sum", np.float64, np.float64, np.int64](s, c, o, n)
            be["awkward_reduce_max", np.float64, np.float64, np.int64](mx, c, o, n, -np.inf)
            be["awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64](
                am, c, o, o[:-1].contiguous(), n)
            be["awkward_reduce_count_64", np.int64, np.int64](ct, o, n)
        so, sc = jagged.getitem_jagged_mask(o, c, m)
        outs.append((s, mx, am, ct, so, sc))
    be.synchronize()
    return outs


def batch_specs(narrays, seed, min_lists=1_000, max_lists=20_000):
    """Per array of the batched-workload distribution: (list count, length
    law, law parameter, seed).  List counts log-uniform in [min_lists,
    max_lists]; lengths Poisson(lambda ~ U(1, 32)) or Geometric(0.02) - 1 (a
    seeded fair coin)."""
    rng = np.random.default_rng(seed)
    specs = []
    for a in range(narrays):
        n = int(round(math.exp(rng.uniform(math.log(min_lists), math.log(max_lists)))))
        if rng.random() < 0.5:
            specs.append((n, "poisson", float(rng.uniform(1, 32)), seed * 1_000_003 + a))
        else:
            specs.append((n, "geometric", 0.02, seed * 1_000_003 + a))
    return specs


def spec_bytes(spec):
    """Estimated device bytes of one generated array (content, mask, select
    output, offsets and the five per-list outputs)."""
    n, law, p, _seed = spec
    mean = p if law == "poisson" else (1 - p) / p
    return int(n * mean * 0.95 * 17 + n * 56)


def make_wave(specs, device="cuda"):
    """The arrays of `specs`, generated on the device (5% empty lists, float64
    N(0,1) content, Bernoulli(0.4) mask), each from its own seed."""
    arrays = []
    for n, law, p, seed in specs:
        gen = torch.Generator(device=device).manual_seed(seed)
        if law == "poisson":
            L = torch.poisson(torch.full((n,), p, device=device), generator=gen).to(torch.int64)
        else:
            u = torch.rand(n, device=device, generator=gen).clamp_min(1e-12)
            L = torch.floor(torch.log(u) / math.log(1 - p)).to(torch.int64)
        L[torch.rand(n, device=device, generator=gen) < 0.05] = 0
        off = torch.zeros(n + 1, dtype=torch.int64, device=device)
        torch.cumsum(L, 0, out=off[1:])
        E = int(off[-1].item())
        x = torch.randn(E, dtype=torch.float64, device=device, generator=gen)
        mask = torch.rand(E, device=device, generator=gen) < 0.4
        arrays.append((off, x, mask))
    return Batch(arrays)


def make_batch(narrays, seed, min_lists=1_000, max_lists=20_000, device="cuda"):
    """The batched-workload generator: batch_specs generated on the device."""
    return make_wave(batch_specs(narrays, seed, min_lists, max_lists), device)


def waves(specs, max_bytes):
    """Consecutive groups of specs of at most max_bytes estimated bytes each."""
    out, cur, size = [], [], 0
    for sp in specs:
        b = spec_bytes(sp)
        if cur and size + b > max_bytes:
            out.append(cur)
            cur, size = [], 0
        cur.append(sp)
        size += b
    if cur:
        out.append(cur)
    return out


def time_plain(batch, reps=1):
    torch.cuda.synchronize(batch.device)
    t0 = time.perf_counter()
    for _ in range(reps):
        run_plain(batch)
    torch.cuda.synchronize(batch.device)
    return (time.perf_counter() - t0) / reps * 1e3
