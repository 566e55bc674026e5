"""Drop-in entry points inside a CUDA graph.

The segmented reducers and the list-tile kernels make no host synchronisation
per call (their scratch comes from a stream-ordered pool), so a sequence of
calls captures into one CUDA graph.  Replays must give the eager results bit
for bit, and follow the inputs when they change in place.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_reducers_and_jagged_apply_replay_from_a_cuda_graph():
    import torch

    import awkward_gb300

    be = awkward_gb300.backend()
    rng = np.random.default_rng(31)
    n = 1_000_000
    L = rng.poisson(8, n)
    L[rng.random(n) < 0.01] = 0
    L[4242] = 20_000  # a list crossing warp ranges: the fix-up kernel runs too
    off_h = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    E = int(off_h[-1])
    off = torch.from_numpy(off_h).cuda()
    x = torch.from_numpy(rng.standard_normal(E)).cuda()
    K = np.where(L > 0, rng.poisson(2, n), 0)
    soff_h = np.concatenate([[0], np.cumsum(K)]).astype(np.int64)
    idx_h = np.concatenate([rng.integers(-l, l, k) for l, k in zip(L, K) if k]).astype(np.int64)
    soff, idx = torch.from_numpy(soff_h).cuda(), torch.from_numpy(idx_h).cuda()
    starts, stops = off[:-1].contiguous(), off[1:].contiguous()
    o_sum = torch.empty(n, dtype=torch.float64, device="cuda")
    o_max = torch.empty(n, dtype=torch.float64, device="cuda")
    o_arg = torch.empty(n, dtype=torch.int64, device="cuda")
    t_off = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    t_carry = torch.empty(len(idx_h), dtype=torch.int64, device="cuda")
    k_sum = be["awkward_reduce_sum", np.float64, np.float64, np.int64]
    k_max = be["awkward_reduce_max", np.float64, np.float64, np.int64]
    k_arg = be["awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64]
    k_app = be["awkward_ListArray_getitem_jagged_apply", np.int64, np.int64, np.int64, np.int64,
               np.int64, np.int64, np.int64]

    def run():
        k_sum(o_sum, x, off, n)
        k_max(o_max, x, off, n, -np.inf)
        k_arg(o_arg, x, off, starts, n)
        k_app(t_off, t_carry, soff[:-1], soff[1:], n, idx, len(idx_h), starts, stops, E)

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        run()
    be.synchronize(s)
    eager = [t.clone() for t in (o_sum, o_max, o_arg, t_off, t_carry)]

    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        run()
    for t in (o_sum, o_max, t_off, t_carry):
        t.fill_(123)
    o_arg.fill_(-7)
    g.replay()
    torch.cuda.synchronize()
    for got, exp in zip((o_sum, o_max, o_arg, t_off, t_carry), eager):
        assert torch.equal(got.view(torch.int64) if got.is_floating_point() else got,
                           exp.view(torch.int64) if exp.is_floating_point() else exp)

    # the graph reads the inputs where they are: new values, new results
    x.mul_(-2.0)
    g.replay()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        e_max = torch.empty_like(o_max)
        k_max(e_max, x, off, n, -np.inf)
    be.synchronize(s)
    assert torch.equal(o_max.view(torch.int64), e_max.view(torch.int64))
