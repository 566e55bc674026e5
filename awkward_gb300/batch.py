"""Batched jagged operations: many arrays, one launch per operation, one CUDA graph.

``Batch`` holds A float64 ListOffsetArrays ``(offsets, content)`` with one
jagged boolean mask each (CUDA tensors) and the outputs of

    sum, max, argmax, count (axis=-1)   and   array[mask]

for every array.  ``Batch.plan(order_mode, occupancy_div)`` builds the device
work queue (libawkward_gb300's batch plan); ``Batch.graph(plan)`` captures one
run of every operation in a CUDA graph, and ``graph.replay()`` re-runs it.

``autotune(batch)`` times the plan variants on the batch itself and keeps the
fastest, cached under a signature of the batch's length histogram (counts of
arrays per power-of-two bucket of list count and of mean list length), so
batches with the same shape profile reuse the choice.

``run_plain(batch)`` runs the same operations array by array through the
per-array entry points (awkward's own sequence of calls, with its host
reads of data-dependent sizes) -- the reference the batched outputs equal
bit for bit.
"""

from __future__ import annotations

import ctypes
import math
import time

import numpy as np
import torch

from . import _abi
from .kernel_table import backend

PLAN_VARIANTS = [(0, 1), (1, 1), (1, 2), (0, 2)]  # (order_mode, occupancy_div)
_TUNED = {}


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

    def plan(self, order_mode=1, occupancy_div=1):
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
            order_mode, occupancy_div, self.err.data_ptr())
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


def autotune(batch, reps=5):
    """(order_mode, occupancy_div) of the fastest plan for this batch's shape."""
    sig = batch.signature()
    if sig in _TUNED:
        return _TUNED[sig]
    best, best_ms = None, math.inf
    for variant in PLAN_VARIANTS:
        plan = batch.plan(*variant)
        g = batch.graph(plan)
        g.replay()
        torch.cuda.synchronize(batch.device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            g.replay()
        b.record()
        torch.cuda.synchronize(batch.device)
        ms = a.elapsed_time(b) / reps
        if ms < best_ms:
            best, best_ms = variant, ms
        del g
    _TUNED[sig] = best
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


def make_batch(narrays, seed, min_lists=1_000, max_lists=20_000, device="cuda"):
    """The batched-workload generator: list counts log-uniform in [min_lists,
    max_lists]; per array, lengths Poisson(lambda ~ U(1, 32)) or Geometric(0.02) - 1
    (a seeded fair coin), 5% empty lists; float64 N(0,1) content; mask
    Bernoulli(0.4).  Generated on the device from seeded torch generators."""
    rng = np.random.default_rng(seed)
    arrays = []
    gen = torch.Generator(device=device).manual_seed(seed)
    for _ in range(narrays):
        n = int(round(math.exp(rng.uniform(math.log(min_lists), math.log(max_lists)))))
        if rng.random() < 0.5:
            lam = rng.uniform(1, 32)
            L = torch.poisson(torch.full((n,), lam, device=device), generator=gen).to(torch.int64)
        else:
            u = torch.rand(n, device=device, generator=gen).clamp_min(1e-12)
            L = torch.floor(torch.log(u) / math.log(1 - 0.02)).to(torch.int64)
        L[torch.rand(n, device=device, generator=gen) < 0.05] = 0
        off = torch.zeros(n + 1, dtype=torch.int64, device=device)
        torch.cumsum(L, 0, out=off[1:])
        E = int(off[-1].item())
        x = torch.randn(E, dtype=torch.float64, device=device, generator=gen)
        mask = torch.rand(E, device=device, generator=gen) < 0.4
        arrays.append((off, x, mask))
    return Batch(arrays)


def time_plain(batch, reps=1):
    torch.cuda.synchronize(batch.device)
    t0 = time.perf_counter()
    for _ in range(reps):
        run_plain(batch)
    torch.cuda.synchronize(batch.device)
    return (time.perf_counter() - t0) / reps * 1e3
