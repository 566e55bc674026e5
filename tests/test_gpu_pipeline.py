"""GPU test of the host-buffer reduction with overlapped transfers.

reduce_host (pinned CPU inputs, chunks of lists copied, reduced and copied
back on three streams) must give the results of the device entry points
awkward_reduce_{sum,max,argmax} on the whole array, for any number of chunks,
with empty lists, offsets not starting at 0 and a 2,000,000-element list:
max and argmax bit-identical; sums bit-identical for lists of up to 4096
elements and, for longer lists (whose fixed-point partials depend on how the
lists are split into warp ranges, which the chunking changes), within
4*n*eps*sum|x|.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("chunks", [1, 3, 8, 64])
@pytest.mark.parametrize("kind", ["poisson", "giant"])
def test_reduce_host_matches_device(chunks, kind):
    import torch

    import awkward_gb300
    from awkward_gb300 import pipeline

    rng = np.random.default_rng(chunks)
    L = rng.poisson(8, 300_000)
    L[rng.random(len(L)) < 0.01] = 0
    if kind == "giant":
        L[1000] = 2_000_000
    off = (np.concatenate([[0], np.cumsum(L)]) + 5).astype(np.int64)
    x = rng.standard_normal(int(off[-1]))
    xh = torch.from_numpy(x).pin_memory()
    oh = torch.from_numpy(off).pin_memory()
    s, m, a = pipeline.reduce_host(xh, oh, chunks=chunks)
    torch.cuda.current_stream().synchronize()
    be = awkward_gb300.backend()
    n = len(L)
    dx, do = xh.cuda(), oh.cuda()
    es = torch.empty(n, dtype=torch.float64, device="cuda")
    em = torch.empty(n, dtype=torch.float64, device="cuda")
    ea = torch.empty(n, dtype=torch.int64, device="cuda")
    be["awkward_reduce_sum", np.float64, np.float64, np.int64](es, dx, do, n)
    be["awkward_reduce_max", np.float64, np.float64, np.int64](em, dx, do, n, -np.inf)
    be["awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64](ea, dx, do,
                                                                          do[:-1].contiguous(), n)
    be.synchronize()
    es = es.cpu()
    short = torch.from_numpy(L <= 4096)
    assert torch.equal(s[short].view(torch.int64), es[short].view(torch.int64))
    absx = np.concatenate([[0.0], np.cumsum(np.abs(x))])
    bound = 4 * np.maximum(L, 1) * np.finfo(np.float64).eps * (absx[off[1:]] - absx[off[:-1]])
    assert np.all(np.abs(s.numpy() - es.numpy()) <= bound)
    assert torch.equal(m.view(torch.int64), em.cpu().view(torch.int64))
    assert torch.equal(a, ea.cpu())
