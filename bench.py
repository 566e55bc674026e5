"""Benchmark of the GB300 jagged hot path (one JSON line on rank 0).

Headline workload (the configuration the segmented-reduce metric is quoted
on): ak.sum, ak.max and ak.argmax(axis=-1) kernels over a ListOffsetArray of
10,000,000 lists, lengths ~ Poisson(8) with 1% forced empty, int64 offsets
from 0, float64 content ~ N(0,1), seed 0 (about 80M elements, 714 MB of
inputs: larger than the 129 MB L2, so no flush is needed between steps).
One step = the three reducer launches (awkward_reduce_sum_float64_float64_64,
awkward_reduce_max_float64_float64_64, awkward_reduce_argmax_float64_64).

value  = algorithmic bytes of the step / device time (GB/s), inputs resident;
e2e    = the same bytes / time through the C ABI from pinned HOST buffers:
         per step H2D of content+offsets, the three kernels, D2H of the three
         outputs;
roofline = the slowest of the three reducers, algorithmic bytes per launch
         (8E + 8(N+1) + 8N) / its CUDA-event duration, against the measured
         HBM copy bandwidth in MEASURED_PEAKS.json.

``--impl reference`` times awkward's CPU reducers (the compiled awkward-cpp
kernels when present, else the C restatement in oracle/) on all host cores
over the same workload.  ``--gpus N`` (torchrun) runs N independent shards,
one per rank, with no data-path collective (weak scaling).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

N_LISTS = 10_000_000
METRIC = "segmented-reduce GB/s (ak.sum+ak.max+ak.argmax axis=-1, float64)"
UNIT = "GB/s"


def make_c1(n, seed):
    """C1 inputs: Poisson(8) lengths, 1% empty, float64 N(0,1) content."""
    rng = np.random.default_rng(seed)
    L = rng.poisson(8, n).astype(np.int64)
    L[rng.random(n) < 0.01] = 0
    off = np.empty(n + 1, np.int64)
    off[0] = 0
    np.cumsum(L, out=off[1:])
    x = rng.standard_normal(int(off[-1]))
    return off, x


def make_c1_shard(n, rank, world):
    """This rank's shard of one global C1 array of world * n lists.

    The global list lengths come from seed 0 on every rank, the shard is the
    rank's balanced list range (awkward_gb300.shard.local_shard's bounds), and
    its content is drawn from a per-rank seed.  Returns (local offsets from 0,
    content, global offsets slice of the shard, first global list).  With
    world == 1 this is exactly make_c1(n, 0).
    """
    if world == 1:
        off, x = make_c1(n, 0)
        return off, x, off, 0
    from awkward_gb300 import shard

    rng = np.random.default_rng(0)
    N = n * world
    L = rng.poisson(8, N).astype(np.int64)
    L[rng.random(N) < 0.01] = 0
    goff = np.empty(N + 1, np.int64)
    goff[0] = 0
    np.cumsum(L, out=goff[1:])
    b = shard.shard_bounds(goff, world)
    l0, l1 = int(b[rank]), int(b[rank + 1])
    gslice = goff[l0:l1 + 1]
    local = gslice - gslice[0]
    x = np.random.default_rng(1000 + rank).standard_normal(int(local[-1]))
    return local, x, gslice, l0


def algorithmic_bytes(n, e):
    """Per reducer launch: content + offsets read, one 8-byte result per list."""
    return 8 * e + 8 * (n + 1) + 8 * n


def measured_peak():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile(op, n_lists):
    """DRAM bytes per launch of reducer `op` from the committed ncu summary.

    profiles/seg_reduce_traffic.txt holds ``<op> <lists> <dram bytes per launch>``
    lines measured with ncu on a smaller C1 case; the figure is scaled by the
    list count (traffic grows in proportion to the lists processed).
    """
    path = os.path.join(HERE, "profiles", "seg_reduce_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split("#", 1)[0].split()
                if len(parts) == 3 and parts[0] == op:
                    return int(round(int(parts[2]) * n_lists / int(parts[1])))
    except (OSError, ValueError):
        return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.tmp is None:
            return None
        try:
            rows = [r.split(",") for r in open(self.tmp.name).read().strip().splitlines() if r]
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup(n_gpus):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    return rank, world, local


def reduce_max(x):
    import torch

    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist

        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def barrier():
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist

        dist.barrier()


def cpu_reduce_step(lib_kind, off, x, outs, threads):
    import oracle

    n = len(off) - 1
    oracle.parallel_reduce("awkward_reduce_sum_float64_float64_64", outs[0], x, off, n, threads)
    oracle.parallel_reduce("awkward_reduce_max_float64_float64_64", outs[1], x, off, n, threads,
                           identity=-np.inf)
    oracle.parallel_reduce("awkward_reduce_argmax_float64_64", outs[2], x, off, n, threads)


def _time_cpu_steps(off, x, threads, target_s):
    n = len(off) - 1
    outs = [np.empty(n), np.empty(n), np.empty(n, np.int64)]
    cpu_reduce_step("port", off, x, outs, threads)  # warm
    t0 = time.perf_counter()
    reps = 0
    while True:
        cpu_reduce_step("port", off, x, outs, threads)
        reps += 1
        if time.perf_counter() - t0 > target_s:
            break
    return (time.perf_counter() - t0) / reps, reps


def cpu_baseline(off, x, target_s=6.0):
    """The C restatement of awkward-cpp's reducers on the full workload:
    on all host cores (pthreads over list ranges), and on one core (awkward-cpp
    itself is single-threaded: its CMakeLists.txt builds the CPU kernels with
    no threading)."""
    threads = os.cpu_count() or 1
    n = len(off) - 1
    nbytes = 3 * algorithmic_bytes(n, len(x))
    dt, reps = _time_cpu_steps(off, x, threads, target_s)
    dt1, reps1 = _time_cpu_steps(off, x, 1, target_s)
    return {"value": round(nbytes / dt / 1e9, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"full workload: {n} C1 lists (Poisson(8), float64), sum+max+argmax, "
                      f"{reps} steps of {dt*1e3:.1f} ms; awkward-cpp restated in oracle/",
            "single_core": {"value": round(nbytes / dt1 / 1e9, 3), "unit": UNIT, "cores": 1,
                            "ms_per_step": round(dt1 * 1e3, 2), "steps": reps1},
            "ms_per_step": round(dt * 1e3, 2)}


def c1_config(n, e, world):
    """The `config` object of both arms (same keys and values for one workload)."""
    return {"workload": f"C1 reducers @ {n} lists Poisson(8) float64 (sum+max+argmax)",
            "lists_per_gpu": n, "elements_per_gpu": e,
            "l2": f"inputs {(8 * e + 8 * (n + 1)) / 1e6:.0f} MB vs 129 MB L2: "
                  + ("larger, no flush needed" if 8 * e + 8 * (n + 1) > 129e6
                     else "SMALLER: timings include L2 reuse"),
            "parallelism": f"{world} independent shard(s), no collective"}


def c1_parity(off, x, got_sum, got_max, got_arg):
    """The timed outputs against the oracle on the full input: argmax and max
    bit for bit (C restatement over all host cores), the float sum's error
    figures against the FP64 compensated-sum oracle (bound 4*n*eps*sum|x|)."""
    import oracle

    threads = os.cpu_count() or 1
    n = len(off) - 1
    e_max, e_arg = np.empty(n), np.empty(n, np.int64)
    oracle.parallel_reduce("awkward_reduce_max_float64_float64_64", e_max, x, off, n, threads,
                           identity=-np.inf)
    oracle.parallel_reduce("awkward_reduce_argmax_float64_64", e_arg, x, off, n, threads)
    rep = oracle.sum_error_report(got_sum, x, off, nthreads=threads)
    return {"argmax_bit_exact": bool(np.array_equal(got_arg, e_arg)),
            "max_bit_exact": bool(np.array_equal(got_max.view(np.int64), e_max.view(np.int64))),
            "sum_err": {k: (float(f"{v:.4g}") if isinstance(v, float) else v) for k, v in rep.items()},
            "sum_bound": "|gpu - compensated| <= 4*n*eps*sum|x| per list; ratio = err/(n*eps*sum|x|)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t = []
    off, x = make_c1(args.lists, 0)
    n = len(off) - 1
    threads = os.cpu_count() or 1
    outs = [np.empty(n), np.empty(n), np.empty(n, np.int64)]
    for _ in range(args.warmup):
        cpu_reduce_step("port", off, x, outs, threads)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_reduce_step("port", off, x, outs, threads)
        t.append(time.perf_counter() - t0)
    dt = sum(t) / len(t)
    gbs = 3 * algorithmic_bytes(n, len(x)) / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded C1 generator)",
            "config": c1_config(n, int(len(x)), int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": round(gbs, 3), "unit": UNIT, "cores": threads,
                             "kind": "port",
                             "sample": f"full workload ({n} lists) per step, pthreads over "
                                       f"list ranges; awkward-cpp restated in oracle/"},
            "e2e": {"value": round(gbs, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _time_ms(fn, reps, stream):
    """Mean device time of fn() over reps launches (CUDA events on `stream`)."""
    import torch

    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def measure_c3(be, dev, reps, warmup, n_lists=5_000_000, n3_lists=1_000_000):
    """ak.combinations(axis=1): n=2 on lists of min(Poisson(6), 40), n=3 on Poisson(4).

    Per configuration: combinations_length (tuple counts, offsets, total)
    then combinations (the n carries), inputs resident; tuples/s over both
    kernels; algorithmic bytes of the fill 16N + 8(N+1) + 8nP.
    """
    import torch

    res = {}
    stream = torch.cuda.current_stream(dev)
    for n, nl, lam, cap, seed in ((2, n_lists, 6, 40, 3), (3, n3_lists, 4, None, 4)):
        rng = np.random.default_rng(seed)
        L = rng.poisson(lam, nl)
        if cap:
            L = np.minimum(L, cap)
        off = torch.from_numpy(np.concatenate([[0], np.cumsum(L)]).astype(np.int64)).to(dev)
        st, sp = off[:-1].contiguous(), off[1:].contiguous()
        tot = torch.empty(1, dtype=torch.int64, device=dev)
        too = torch.empty(nl + 1, dtype=torch.int64, device=dev)
        kl = be["awkward_ListArray_combinations_length", np.int64, np.int64, np.int64, np.int64]
        kc = be["awkward_ListArray_combinations", np.int64, np.int64, np.int64, np.int64, np.int64]
        kl(tot, too, n, False, st, sp, nl)
        be.synchronize()
        P = int(tot.item())
        rows = [torch.empty(P, dtype=torch.int64, device=dev) for _ in range(n)]
        ti = torch.empty(n, dtype=torch.int64, device=dev)
        fi = torch.zeros(n, dtype=torch.int64, device=dev)
        for _ in range(max(warmup, 3)):
            kl(tot, too, n, False, st, sp, nl)
            kc(rows, ti, fi, n, False, st, sp, nl)
        be.synchronize()
        t_len = _time_ms(lambda: kl(tot, too, n, False, st, sp, nl), reps, stream)
        t_fill = _time_ms(lambda: kc(rows, ti, fi, n, False, st, sp, nl), reps, stream)
        be.synchronize()
        fill_bytes = 16 * nl + 8 * (nl + 1) + 8 * n * P
        res[f"n{n}"] = {
            "lists": nl, "tuples": P,
            "tuples_per_s": round(P / ((t_len + t_fill) * 1e-3), 1),
            "length_us": round(t_len * 1e3, 1), "fill_us": round(t_fill * 1e3, 1),
            "fill_gbs": round(fill_bytes / (t_fill * 1e-3) / 1e9, 1),
            "lengths": f"min(Poisson({lam}), {cap})" if cap else f"Poisson({lam})",
        }
        del rows
    return res


def measure_c2(be, dev, reps, warmup, n_lists=10_000_000):
    """Jagged slicing at 10M lists (Poisson(8), float32 content ~ Exp(1)*20, seed 1):
    array[mask] (Bernoulli(0.4) jagged mask), array[idx] (per list Poisson(2)
    int64 indices in [-len, len)), and [..., 1:] on a two-level array (10M outer
    lists of Poisson(4) inner lists of Poisson(6)).  Device time of each chain's
    kernels with outputs pre-sized (the sizes awkward reads back are read once
    before timing)."""
    import torch

    from awkward_gb300 import _abi, jagged

    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    gen = torch.Generator(device=dev).manual_seed(1)
    L = torch.poisson(torch.full((n_lists,), 8.0, device=dev), generator=gen).to(torch.int64)
    off = torch.zeros(n_lists + 1, dtype=torch.int64, device=dev)
    torch.cumsum(L, 0, out=off[1:])
    E = int(off[-1].item())
    x = (torch.empty(E, device=dev).exponential_(1.0, generator=gen) * 20).to(torch.float32)
    mask = torch.rand(E, device=dev, generator=gen) < 0.4
    K = torch.where(L > 0, torch.poisson(torch.full((n_lists,), 2.0, device=dev), generator=gen),
                    torch.zeros((), device=dev)).to(torch.int64)
    ioff = torch.zeros(n_lists + 1, dtype=torch.int64, device=dev)
    torch.cumsum(K, 0, out=ioff[1:])
    owner = torch.repeat_interleave(torch.arange(n_lists, device=dev), K)
    Lk = L[owner]
    idx = (torch.rand(owner.numel(), device=dev, generator=gen) * (2 * Lk)).to(torch.int64) - Lk
    err = torch.full((1,), -1, dtype=torch.int64, device=dev)
    f_m2i = _abi.ext_cfunc("awkward_gb300_jagged_mask_to_index")
    f_take = _abi.ext_cfunc("awkward_gb300_take")
    k_apply = be["awkward_ListArray_getitem_jagged_apply", np.int64, np.int64, np.int64, np.int64,
                 np.int64, np.int64, np.int64]
    starts, stops = off[:-1].contiguous(), off[1:].contiguous()
    # mask chain buffers
    m_ioff = torch.empty(n_lists + 1, dtype=torch.int64, device=dev)
    m_idx = torch.empty(E, dtype=torch.int64, device=dev)
    f_m2i(m_ioff.data_ptr(), m_idx.data_ptr(), mask.data_ptr(), off.data_ptr(), n_lists,
          err.data_ptr(), sp)
    Km = int(m_ioff[-1].item())
    m_ist, m_isp = m_ioff[:-1].contiguous(), m_ioff[1:].contiguous()
    m_too = torch.empty(n_lists + 1, dtype=torch.int64, device=dev)
    m_carry = torch.empty(Km, dtype=torch.int64, device=dev)
    m_out = torch.empty(Km, dtype=torch.float32, device=dev)

    def mask_chain():
        f_m2i(m_ioff.data_ptr(), m_idx.data_ptr(), mask.data_ptr(), off.data_ptr(), n_lists,
              err.data_ptr(), sp)
        k_apply(m_too, m_carry, m_ist, m_isp, n_lists, m_idx[:Km], Km, starts, stops, E)
        f_take(m_out.data_ptr(), x.data_ptr(), 4, m_carry.data_ptr(), Km, E, 0, err.data_ptr(), sp)

    f_sel = _abi.ext_cfunc("awkward_gb300_jagged_mask_select")
    s_off = torch.empty(n_lists + 1, dtype=torch.int64, device=dev)
    s_out = torch.empty(E, dtype=torch.float32, device=dev)

    def mask_one_pass():
        f_sel(s_off.data_ptr(), s_out.data_ptr(), None, mask.data_ptr(), off.data_ptr(),
              x.data_ptr(), 4, n_lists, err.data_ptr(), sp)

    Ki = idx.numel()
    i_ist, i_isp = ioff[:-1].contiguous(), ioff[1:].contiguous()
    i_too = torch.empty(n_lists + 1, dtype=torch.int64, device=dev)
    i_carry = torch.empty(Ki, dtype=torch.int64, device=dev)
    i_out = torch.empty(Ki, dtype=torch.float32, device=dev)

    def index_chain():
        k_apply(i_too, i_carry, i_ist, i_isp, n_lists, idx, Ki, starts, stops, E)
        f_take(i_out.data_ptr(), x.data_ptr(), 4, i_carry.data_ptr(), Ki, E, 0, err.data_ptr(), sp)

    f_isel = _abi.ext_cfunc("awkward_gb300_jagged_index_select")
    j_too = torch.empty(n_lists + 1, dtype=torch.int64, device=dev)
    j_out = torch.empty(Ki, dtype=torch.float32, device=dev)

    def index_one_pass():
        f_isel(j_too.data_ptr(), j_out.data_ptr(), None, ioff.data_ptr(), idx.data_ptr(), Ki,
               off.data_ptr(), x.data_ptr(), 4, E, n_lists, err.data_ptr(), sp)

    Lo = torch.poisson(torch.full((n_lists,), 4.0, device=dev), generator=gen).to(torch.int64)
    ninner = int(Lo.sum().item())
    Li = torch.poisson(torch.full((ninner,), 6.0, device=dev), generator=gen).to(torch.int64)
    inner = torch.zeros(ninner + 1, dtype=torch.int64, device=dev)
    torch.cumsum(Li, 0, out=inner[1:])
    E2 = int(inner[-1].item())
    x2 = (torch.empty(E2, device=dev).exponential_(1.0, generator=gen) * 20).to(torch.float32)
    in_st, in_sp = inner[:-1].contiguous(), inner[1:].contiguous()
    k_cl = be["awkward_ListArray_getitem_next_range_carrylength", np.int64, np.int64, np.int64]
    k_nr = be["awkward_ListArray_getitem_next_range", np.int64, np.int64, np.int64, np.int64]
    cl = torch.empty(1, dtype=torch.int64, device=dev)
    k_cl(cl, in_st, in_sp, ninner, 1, jagged.SLICE_NONE, 1)
    be.synchronize()
    Kr = int(cl.item())
    r_off = torch.empty(ninner + 1, dtype=torch.int64, device=dev)
    r_carry = torch.empty(Kr, dtype=torch.int64, device=dev)
    r_out = torch.empty(Kr, dtype=torch.float32, device=dev)

    def range_chain():
        k_cl(cl, in_st, in_sp, ninner, 1, jagged.SLICE_NONE, 1)
        k_nr(r_off, r_carry, in_st, in_sp, ninner, 1, jagged.SLICE_NONE, 1)
        f_take(r_out.data_ptr(), x2.data_ptr(), 4, r_carry.data_ptr(), Kr, E2, 0, err.data_ptr(), sp)

    res = {}
    # algorithmic bytes: mask 1B/elem + offsets 8(N+1) read; index offsets 8(N+1) + index 8K
    # written and read; apply 32N + 16K + 8(N+1); take 8K carry + 4K gather + 4K out
    N = n_lists
    byts = {
        "mask": (E + 8 * (N + 1)) + (8 * (N + 1) + 8 * Km) + (32 * N + 16 * Km + 8 * (N + 1))
        + 16 * Km,
        "index": (32 * N + 16 * Ki + 8 * (N + 1)) + 16 * Ki,
        "range": (16 * ninner + 8) + (16 * ninner + 8 * (ninner + 1) + 8 * Kr) + 16 * Kr,
        # one pass: mask and offsets read, the content read once, new offsets and
        # the selected content written
        "mask_one_pass": E + 8 * (N + 1) + 4 * E + 8 * (N + 1) + 4 * Km,
        # one pass: index offsets, offsets and the index read, the content gathered
        # once, new offsets and the gathered content written (no carry)
        "index_one_pass": 24 * (N + 1) + 8 * Ki + 4 * Ki + 4 * Ki,
    }
    for name, fn, nl in (("mask", mask_chain, N), ("index", index_chain, N),
                         ("range", range_chain, N), ("mask_one_pass", mask_one_pass, N),
                         ("index_one_pass", index_one_pass, N)):
        for _ in range(max(warmup, 3)):
            fn()
        be.synchronize()
        ms = _time_ms(fn, reps, stream)
        be.synchronize()
        res[name] = {"ms": round(ms, 4), "lists_per_s": round(nl / (ms * 1e-3), 1),
                     "gbs": round(byts[name] / (ms * 1e-3) / 1e9, 1)}
    res["mask"]["kernels"] = "mask_to_index + jagged_apply + take (float32)"
    res["index"]["kernels"] = "jagged_apply + take (float32)"
    res["range"]["kernels"] = "next_range_carrylength + next_range + take (float32)"
    res["mask_one_pass"]["kernels"] = ("awkward_gb300_jagged_mask_select: array[mask] in one "
                                       "kernel (same offsets and content as the chain)")
    res["index_one_pass"]["kernels"] = ("awkward_gb300_jagged_index_select: array[idx] in one "
                                        "kernel (same offsets and content as the chain)")
    res["sizes"] = {"lists": N, "elements": E, "selected": Km, "indices": Ki,
                    "inner_lists": ninner, "inner_elements": E2, "range_kept": Kr}
    return res


def measure_c4(dev, narrays=4096, min_lists=1_000, max_lists=20_000, reps=5, full=True):
    """Batched uneven workload: sum/max/argmax/count(axis=-1) + array[mask] of
    `narrays` float64 arrays, lengths Poisson(U(1,32)) or Geometric(0.02) per
    array, 5% empty lists, Bernoulli(0.4) masks, generated on the device from
    per-array seeds.  Batched: one CUDA graph replay of an autotuned plan;
    plain: the per-array entry points array by array (wall time, host reads
    included).

    scaled: list counts log-uniform in [min_lists, max_lists] (one resident
    batch).  full: the configured range [1e3, 2e6] (about 280 GB of content),
    run as resident waves of at most 60 GB generated on the device, one plan
    and one graph per wave (knobs tuned on the first wave); times add up over
    the waves."""
    import torch

    from awkward_gb300 import batch

    def one(b, knobs, reps):
        plan = b.plan(knobs)
        g = b.graph(plan)
        g.replay()
        torch.cuda.synchronize(dev)
        ms_b = _time_ms(g.replay, reps, torch.cuda.current_stream(dev))
        b.check_errors()
        batch.run_plain(b)  # warm the per-array path (pools, kernel table)
        ms_p = batch.time_plain(b, reps=1)
        del g
        return ms_b, ms_p, int(b.nelements.sum()), int(b.nlists.sum())

    def nbytes(E, N):
        return 3 * (8 * E + 16 * N) + (8 * E + E + 16 * N) + 8 * int(0.4 * E)

    res = {}
    b = batch.make_batch(narrays, seed=4, min_lists=min_lists, max_lists=max_lists, device=dev)
    t0 = time.perf_counter()
    knobs = batch.autotune(b, reps=3)
    tune_s = time.perf_counter() - t0
    ms_b, ms_p, E, N = one(b, knobs, reps)
    b.close()
    del b
    res["scaled"] = {"arrays": narrays, "lists": N, "elements": E,
                     "list_counts": f"log-uniform [{min_lists}, {max_lists}]",
                     "knobs": knobs.__dict__, "tune_s": round(tune_s, 2),
                     "batched_ms": round(ms_b, 3), "plain_ms": round(ms_p, 1),
                     "speedup": round(ms_p / ms_b, 1),
                     "batched_gbs": round(nbytes(E, N) / (ms_b * 1e-3) / 1e9, 1)}
    if full:
        specs = batch.batch_specs(narrays, seed=4, min_lists=1_000, max_lists=2_000_000)
        tot_b = tot_p = 0.0
        E = N = 0
        fknobs = None
        ws = batch.waves(specs, 60e9)
        t0 = time.perf_counter()
        for w in ws:
            b = batch.make_wave(w, device=dev)
            if fknobs is None:
                fknobs = batch.autotune(b, reps=2)
            mb, mp, e, nl = one(b, fknobs, 3)
            tot_b += mb
            tot_p += mp
            E += e
            N += nl
            b.close()
            del b
            torch.cuda.empty_cache()
        res["full"] = {"arrays": narrays, "lists": N, "elements": E, "waves": len(ws),
                       "list_counts": "log-uniform [1000, 2000000]", "knobs": fknobs.__dict__,
                       "batched_ms": round(tot_b, 2), "plain_ms": round(tot_p, 1),
                       "speedup": round(tot_p / tot_b, 2),
                       "batched_gbs": round(nbytes(E, N) / (tot_b * 1e-3) / 1e9, 1),
                       "wall_s": round(time.perf_counter() - t0, 1)}
    return res


def measure_c5(dev, reps, warmup, n_lists=4_000_000):
    """Differentiable ops at 4M lists, Poisson(16), float32: forward + backward
    of segmented sum, max and jagged softmax (256 MB activation budget: the
    softmax backward recomputes max and normaliser).

    fwd_bwd_ms: one step through the public API (torch.autograd, Python
    included; for short kernels the host can be the bound).  kernels_ms: the
    same kernels launched back to back through the C ABI (the reducers, then
    the backward kernel), the device time that the roofline fraction uses."""
    import torch

    import awkward_gb300
    from awkward_gb300 import _abi
    from awkward_gb300 import autograd as ag

    be = awkward_gb300.backend()
    gen = torch.Generator(device=dev).manual_seed(5)
    L = torch.poisson(torch.full((n_lists,), 16.0, device=dev), generator=gen).to(torch.int64)
    off = torch.zeros(n_lists + 1, dtype=torch.int64, device=dev)
    torch.cumsum(L, 0, out=off[1:])
    E = int(off[-1].item())
    x = torch.randn(E, dtype=torch.float32, device=dev, generator=gen).requires_grad_(True)
    xd = x.detach()
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    st = off[:-1].contiguous()
    out = torch.empty(n_lists, dtype=torch.float32, device=dev)
    arg = torch.empty(n_lists, dtype=torch.int64, device=dev)
    gx = torch.empty(E, dtype=torch.float32, device=dev)
    y = torch.empty(E, dtype=torch.float32, device=dev)
    k_sum = be["awkward_reduce_sum", np.float32, np.float32, np.int64]
    k_max = be["awkward_reduce_max", np.float32, np.float32, np.int64]
    k_arg = be["awkward_reduce_argmax", np.int64, np.float32, np.int64, np.int64]
    f = lambda name: _abi.ext_cfunc(name)
    res = {}
    for name, fn in (("sum", ag.segment_sum), ("max", ag.segment_max),
                     ("softmax", ag.jagged_softmax)):
        yv = fn(x, off)
        g = torch.randn(yv.shape, dtype=torch.float32, device=dev, generator=gen)

        def step():
            x.grad = None
            fn(x, off).backward(g)

        if name == "sum":
            def kernels():
                k_sum(out, xd, off, n_lists)
                f("awkward_gb300_segment_sum_backward_float32")(
                    gx.data_ptr(), g.data_ptr(), off.data_ptr(), n_lists, E, sp)
        elif name == "max":
            def kernels():
                k_max(out, xd, off, n_lists, -np.inf)
                k_arg(arg, xd, off, st, n_lists)
                f("awkward_gb300_segment_max_backward_float32")(
                    gx.data_ptr(), g.data_ptr(), arg.data_ptr(), E, n_lists, sp)
        else:
            def kernels():
                f("awkward_gb300_jagged_softmax_forward_float32")(
                    y.data_ptr(), xd.data_ptr(), off.data_ptr(), n_lists, E, sp)
                f("awkward_gb300_jagged_softmax_backward_float32")(
                    gx.data_ptr(), g.data_ptr(), xd.data_ptr(), None, off.data_ptr(), n_lists,
                    E, sp)

        for fn_ in (step, kernels):
            for _ in range(max(warmup, 3)):
                fn_()
        torch.cuda.synchronize(dev)
        ms = _time_ms(step, reps, stream)
        kms = _time_ms(kernels, reps, stream)
        be.synchronize()
        nbytes = c5_bytes(name, n_lists, E, 4)
        gbs = nbytes / (kms * 1e-3) / 1e9
        res[name] = {"fwd_bwd_ms": round(ms, 4), "kernels_ms": round(kms, 4),
                     "algorithmic_bytes": nbytes, "gbs": round(gbs, 1),
                     "frac": round(gbs / measured_peak()[0], 4),
                     "api_gbs": round(nbytes / (ms * 1e-3) / 1e9, 1)}
    res["sizes"] = {"lists": n_lists, "elements": E}
    res["bytes"] = ("forward + backward, each value read or written once per kernel that must "
                    "touch it: sum 8E+24N+16; max 12E+40N+16; softmax 20E+16N+16 (itemsize 4)")
    return res


def c5_bytes(name, n, e, itemsize):
    """Algorithmic bytes of one forward + backward of a C5 operation.

    sum: forward reads x and offsets, writes one value per list; backward
    reads the list gradients and offsets, writes one gradient per element.
    max: forward runs max and argmax (x and offsets each, values + int64
    indices out); backward reads gradients and indices, writes every element
    gradient.  softmax: forward reads x, writes y; backward (recomputing the
    maxima and normalisers from x) reads gradient and x, writes the input
    gradient; offsets read by each kernel.
    """
    off = 8 * (n + 1)
    if name == "sum":
        return (itemsize * e + off + itemsize * n) + (itemsize * n + off + itemsize * e)
    if name == "max":
        return ((itemsize * e + off + itemsize * n) + (itemsize * e + off + 8 * n)
                + (itemsize * n + 8 * n + itemsize * e))
    if name == "softmax":
        return (2 * itemsize * e + off) + (3 * itemsize * e + off)
    raise KeyError(name)


def measure_fused(be, dev, reps, warmup, n_lists=10_000_000):
    """ak.sum(x * y, axis=-1) and ak.max(abs(x), axis=-1) on the C1 shape
    (10M lists of Poisson(8), float64 N(0,1) x and y, seed 7): the fused
    entry point against the two-kernel chain an unfused caller runs (torch's
    elementwise kernel materialising the mapped values, then the reducer).
    Algorithmic bytes: fused 16E (sum) or 8E (max) + 8(N+1) + 8N; the chain
    adds the mapped array written and read back (16E)."""
    import torch

    from awkward_gb300.fused import segment_reduce

    stream = torch.cuda.current_stream(dev)
    off_h, x_h = make_c1(n_lists, 7)
    n, E = len(off_h) - 1, len(x_h)
    off = torch.from_numpy(off_h).to(dev)
    x = torch.from_numpy(x_h).to(dev)
    y = torch.randn(E, dtype=torch.float64, device=dev,
                    generator=torch.Generator(device=dev).manual_seed(7))
    out = torch.empty(n, dtype=torch.float64, device=dev)
    tmp = torch.empty_like(x)
    k_sum = be["awkward_reduce_sum", np.float64, np.float64, np.int64]
    k_max = be["awkward_reduce_max", np.float64, np.float64, np.int64]
    cases = {
        "sum_x_times_y": (lambda: segment_reduce(x, off, "x*y", y, "sum", out=out),
                          lambda: (torch.mul(x, y, out=tmp), k_sum(out, tmp, off, n)), 16),
        "max_abs_x": (lambda: segment_reduce(x, off, "abs", None, "max", out=out),
                      lambda: (torch.abs(x, out=tmp), k_max(out, tmp, off, n, -np.inf)), 8),
    }
    res = {}
    for name, (fused, chain, ebytes) in cases.items():
        for fn in (fused, chain):
            for _ in range(max(warmup, 3)):
                fn()
        be.synchronize()
        t_f = _time_ms(fused, reps, stream)
        t_c = _time_ms(chain, reps, stream)
        be.synchronize()
        nb = ebytes * E + 8 * (n + 1) + 8 * n
        res[name] = {"fused_ms": round(t_f, 4), "chain_ms": round(t_c, 4),
                     "speedup": round(t_c / t_f, 2), "fused_gbs": round(nb / (t_f * 1e-3) / 1e9, 1),
                     "fused_frac": round(nb / (t_f * 1e-3) / 1e9 / measured_peak()[0], 4),
                     "chain_bytes": nb + 16 * E}
    res["sizes"] = {"lists": n, "elements": E}
    return res


def measure_sort(be, dev, reps, warmup, n_lists=10_000_000):
    """ak.argsort / ak.sort(axis=-1) on float64: the C1 shape (10M lists of
    Poisson(8)) and a wide shape (2,000 lists of Poisson(40,000), the merged
    path for segments past 2048).  Device time per call, inputs resident;
    algorithmic bytes 8E read + 8(N+1) offsets + 8E written."""
    import torch

    res = {}
    stream = torch.cuda.current_stream(dev)
    for tag, nl, lam in (("c1_shape", n_lists, 8.0), ("wide", max(n_lists // 5000, 1), 40_000.0)):
        gen = torch.Generator(device=dev).manual_seed(11)
        L = torch.poisson(torch.full((nl,), lam, device=dev), generator=gen).to(torch.int64)
        off = torch.zeros(nl + 1, dtype=torch.int64, device=dev)
        torch.cumsum(L, 0, out=off[1:])
        E = int(off[-1].item())
        x = torch.randn(E, dtype=torch.float64, device=dev, generator=gen)
        idx = torch.empty(E, dtype=torch.int64, device=dev)
        srt = torch.empty(E, dtype=torch.float64, device=dev)
        k_arg = be.by_name("awkward_argsort_float64_int64")
        k_srt = be.by_name("awkward_sort_float64")
        for _ in range(max(warmup, 3)):
            k_arg(idx, x, E, off, nl + 1, True, True)
            k_srt(srt, x, E, off, nl + 1, True, True)
        be.synchronize()
        t_arg = _time_ms(lambda: k_arg(idx, x, E, off, nl + 1, True, True), reps, stream)
        t_srt = _time_ms(lambda: k_srt(srt, x, E, off, nl + 1, True, True), reps, stream)
        be.synchronize()
        nbytes = 16 * E + 8 * (nl + 1)
        res[tag] = {"lists": nl, "elements": E, "argsort_ms": round(t_arg, 4),
                    "sort_ms": round(t_srt, 4),
                    "argsort_gelem_s": round(E / (t_arg * 1e-3) / 1e9, 2),
                    "argsort_gbs": round(nbytes / (t_arg * 1e-3) / 1e9, 1)}
        del x, idx, srt
    return res


def measure_nonlocal(be, dev, reps, warmup, n_rows=10_000_000):
    """Reductions above the innermost axis, the kernel sequence awkward runs
    (listoffsetarray.py _reduce_next, non-local branch): maxcount_offsetscopy,
    preparenext, the content carry, the segmented sum over the next offsets and
    outstartsstops.  axis0: ak.sum(x, axis=0) of 10M rows of Poisson(8)
    float64 (one outer bin); axis1: ak.sum(x, axis=1) of a 3-level array, 1M
    outer lists of Poisson(8) rows of Poisson(4).  Device time of the whole
    sequence including its host reads of the sizes; elements/s."""
    import torch

    from awkward_gb300 import _abi

    f_take = _abi.ext_cfunc("awkward_gb300_take")
    k_mc = be.by_name("awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64")
    k_pn = be.by_name("awkward_ListOffsetArray_reduce_nonlocal_preparenext_64")
    k_os = be.by_name("awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64")
    k_sum = be["awkward_reduce_sum", np.float64, np.float64, np.int64]
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    res = {}
    for tag, nbins, lam_rows, lam_len in (("axis0", 1, None, 8.0),
                                          ("axis1", max(n_rows // 10, 1), 8.0, 4.0)):
        gen = torch.Generator(device=dev).manual_seed(13)
        if lam_rows is None:
            R = torch.full((1,), n_rows, dtype=torch.int64, device=dev)
        else:
            R = torch.poisson(torch.full((nbins,), lam_rows, device=dev), generator=gen).to(torch.int64)
        outer = torch.zeros(nbins + 1, dtype=torch.int64, device=dev)
        torch.cumsum(R, 0, out=outer[1:])
        nrows = int(outer[-1].item())
        L = torch.poisson(torch.full((nrows,), lam_len, device=dev), generator=gen).to(torch.int64)
        off = torch.zeros(nrows + 1, dtype=torch.int64, device=dev)
        torch.cumsum(L, 0, out=off[1:])
        E = int(off[-1].item())
        x = torch.randn(E, dtype=torch.float64, device=dev, generator=gen)
        mc = torch.empty(1, dtype=torch.int64, device=dev)
        ocopy = torch.empty(nrows + 1, dtype=torch.int64, device=dev)
        k_mc(mc, ocopy, off, nrows)
        be.synchronize()
        M = int(mc.item())
        nb = nbins * M
        carry = torch.empty(E, dtype=torch.int64, device=dev)
        noff = torch.empty(nb + 1, dtype=torch.int64, device=dev)
        mnp = torch.empty(1, dtype=torch.int64, device=dev)
        dist = torch.empty(nb, dtype=torch.int64, device=dev)
        nxt = torch.empty(E, dtype=torch.float64, device=dev)
        out = torch.empty(nb, dtype=torch.float64, device=dev)
        ost = torch.empty(nbins, dtype=torch.int64, device=dev)
        osp = torch.empty(nbins, dtype=torch.int64, device=dev)
        err = torch.full((1,), -1, dtype=torch.int64, device=dev)

        def chain():
            k_mc(mc, ocopy, off, nrows)
            k_pn(carry, noff, E, mnp, dist, nb, ocopy, off, nrows, outer, nbins, M)
            f_take(nxt.data_ptr(), x.data_ptr(), 8, carry.data_ptr(), E, E, 0, err.data_ptr(), sp)
            k_sum(out, nxt, noff, nb)
            k_os(ost, osp, dist, nb, nbins)

        for _ in range(max(warmup, 3)):
            chain()
        be.synchronize()
        t = _time_ms(chain, reps, stream)
        be.synchronize()
        res[tag] = {"outer_bins": nbins, "rows": nrows, "elements": E, "maxcount": M,
                    "chain_ms": round(t, 4), "gelem_s": round(E / (t * 1e-3) / 1e9, 2)}
        del x, carry, nxt
    return res


def run_gb300(args):
    import torch

    import awkward_gb300

    rank, world, local = dist_setup(args.gpus)
    dev = torch.device("cuda", torch.cuda.current_device())
    be = awkward_gb300.backend()
    if args.only == "c2":
        print(json.dumps({"c2_jagged_slicing": measure_c2(be, dev, args.steps, args.warmup,
                                                          args.lists or 10_000_000)}))
        return
    if args.only == "c4":
        print(json.dumps({"c4_batched": measure_c4(dev, narrays=args.lists or 4096,
                                                    full=not args.no_c4_full)}))
        return
    if args.only == "c5":
        print(json.dumps({"c5_autograd": measure_c5(dev, args.steps, args.warmup,
                                                    args.lists or 4_000_000)}))
        return
    if args.only == "sort":
        print(json.dumps({"sort": measure_sort(be, dev, args.steps, args.warmup,
                                               args.lists or 10_000_000)}))
        return
    if args.only == "nonlocal":
        print(json.dumps({"nonlocal_reduce": measure_nonlocal(be, dev, args.steps, args.warmup,
                                                              args.lists or 10_000_000)}))
        return
    if args.only == "fused":
        print(json.dumps({"fused_reduce": measure_fused(be, dev, args.steps, args.warmup,
                                                        args.lists or 10_000_000)}))
        return
    if args.only == "c3":
        n2 = args.lists or 5_000_000
        print(json.dumps({"c3_combinations": measure_c3(be, dev, args.steps, args.warmup, n2,
                                                        max(n2 // 5, 1))}))
        return
    if args.lists is None:
        args.lists = N_LISTS
    k_sum = be["awkward_reduce_sum", np.float64, np.float64, np.int64]
    k_max = be["awkward_reduce_max", np.float64, np.float64, np.int64]
    k_arg = be["awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64]

    off_h, x_h, goff_h, first_list = make_c1_shard(args.lists, rank, world)
    n, e = len(off_h) - 1, len(x_h)
    off = torch.from_numpy(off_h).to(dev)
    x = torch.from_numpy(x_h).to(dev)
    starts = off[:-1].contiguous()
    o_sum = torch.empty(n, dtype=torch.float64, device=dev)
    o_max = torch.empty(n, dtype=torch.float64, device=dev)
    o_arg = torch.empty(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        k_sum(o_sum, x, off, n)
        k_max(o_max, x, off, n, -np.inf)
        k_arg(o_arg, x, off, starts, n)

    for _ in range(max(args.warmup, 3)):
        step()
    be.synchronize()

    # per-kernel durations (CUDA events on the launching stream)
    nk = max(args.steps, 5)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(nk)]
    for i in range(nk):
        ev[i][0].record(stream)
        k_sum(o_sum, x, off, n)
        ev[i][1].record(stream)
        k_max(o_max, x, off, n, -np.inf)
        ev[i][2].record(stream)
        k_arg(o_arg, x, off, starts, n)
        ev[i][3].record(stream)
    torch.cuda.synchronize()
    be.synchronize()
    per = {name: statistics.mean(ev[i][j].elapsed_time(ev[i][j + 1]) for i in range(nk))
           for j, name in enumerate(["sum", "max", "argmax"])}

    # timed region
    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    with sampler:
        time.sleep(0.3)
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            step()
        stop.record(stream)
        torch.cuda.synchronize()
    be.synchronize()
    ms = start.elapsed_time(stop) / args.steps
    ms = reduce_max(ms)
    step_bytes = 3 * algorithmic_bytes(n, e)
    value = world * step_bytes / (ms * 1e-3) / 1e9

    # end to end through the public host-buffer call (pinned host inputs and
    # outputs; chunked transfers overlapped with the reductions)
    from awkward_gb300 import pipeline

    x_pin = torch.from_numpy(x_h).pin_memory()
    off_pin = torch.from_numpy(off_h).pin_memory()
    outs_pin = (torch.empty(n, dtype=torch.float64).pin_memory(),
                torch.empty(n, dtype=torch.float64).pin_memory(),
                torch.empty(n, dtype=torch.int64).pin_memory())
    ws = pipeline.Workspace(n, int(off_h[-1]), device=dev)
    dev_outs = (o_sum.cpu().numpy(), o_max.cpu().numpy(), o_arg.cpu().numpy())
    del x, off, starts  # the workspace holds the device copies

    def e2e_step():
        pipeline.reduce_host(x_pin, off_pin, chunks=args.chunks, workspace=ws, out=outs_pin)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    be.synchronize()
    barrier()
    s2, t2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s2.record(stream)
    for _ in range(args.steps):
        e2e_step()
    t2.record(stream)
    torch.cuda.synchronize()
    be.synchronize()
    ms_e2e = reduce_max(s2.elapsed_time(t2) / args.steps)
    e2e_same = all(np.array_equal(a.numpy().view(np.int64), b.view(np.int64))
                   for a, b in zip(outs_pin, dev_outs))
    e2e_value = world * step_bytes / (ms_e2e * 1e-3) / 1e9

    # the one collective of sharded execution: local offsets rebased by the
    # exclusive prefix of the shards' totals (an allgather over NCCL), which
    # must give the global offsets of this rank's lists
    from awkward_gb300 import shard

    rebased = shard.rebase_offsets(off_h)
    shard_info = {"first_list": first_list, "lists": n, "elements": e,
                  "rebase_ok": bool(reduce_max(0.0 if np.array_equal(rebased, goff_h) else 1.0)
                                    == 0.0)}
    dominant = max(per, key=per.get)
    peak, peak_kind = measured_peak()
    achieved = algorithmic_bytes(n, e) / (per[dominant] * 1e-3) / 1e9
    traffic = traffic_from_profile(dominant, n)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded C1 generator: Poisson(8) lengths, 1% empty, N(0,1))",
        "config": c1_config(n, e, world),
        "per_kernel_ms": {k: round(v, 4) for k, v in per.items()},
        "roofline": {"bound": "hbm", "kernel": f"seg_reduce ({dominant})",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": algorithmic_bytes(n, e)},
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT,
                "h2d_bytes_per_step": int(8 * e + 8 * (n + 1)),
                "d2h_bytes_per_step": int(3 * 8 * n), "ms_per_step": round(ms_e2e, 4),
                "path": f"awkward_gb300.pipeline.reduce_host, {args.chunks} chunks",
                "outputs_equal_device_path": e2e_same},
        "gpu_launches": args.steps * 3 * 2,
        "shard": shard_info,
        "clocks": sampler.summary(),
    }
    if rank == 0 and not args.no_extras:
        line["c3_combinations"] = measure_c3(be, dev, max(args.steps // 2, 5), args.warmup)
        line["c2_jagged_slicing"] = measure_c2(be, dev, max(args.steps // 2, 5), args.warmup)
        line["c5_autograd"] = measure_c5(dev, max(args.steps // 2, 5), args.warmup)
        line["c4_batched"] = measure_c4(dev, full=not args.no_c4_full)
        line["sort"] = measure_sort(be, dev, max(args.steps // 2, 5), args.warmup)
        line["nonlocal_reduce"] = measure_nonlocal(be, dev, max(args.steps // 2, 5), args.warmup)
        line["fused_reduce"] = measure_fused(be, dev, max(args.steps // 2, 5), args.warmup)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["parity"] = c1_parity(off_h, x_h, *dev_outs)
        line["cpu_baseline"] = cpu_baseline(off_h, x_h)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--chunks", type=int, default=8,
                   help="list chunks of the host-buffer (e2e) pipeline")
    p.add_argument("--no-c4-full", action="store_true",
                   help="skip the full-distribution (waves) run of the batched workload")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the secondary workloads (combinations, ...)")
    p.add_argument("--only", default=None, choices=["c2", "c3", "c4", "c5", "sort", "nonlocal", "fused"],
                   help="run one secondary workload alone (profiling); --lists sets its size")
    p.add_argument("--lists", type=int, default=None,
                   help="list count (default: 10M lists for the reducers, 5M for --only c3; "
                        "smaller values are for profiling captures)")
    args = p.parse_args()
    if args.impl == "reference":
        if args.lists is None:
            args.lists = N_LISTS
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
