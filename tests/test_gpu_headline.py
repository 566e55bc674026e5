"""GPU parity on the headline configurations of the segmented reducers.

* 1,000,000 lists, lengths Poisson(8) with 1% forced empty, float64 N(0,1)
  content, seed 0 -- the plain segmented-reduce configuration awkward-cpp runs
  on the CPU;
* 10,000,000 lists of the same distribution, seed 0 -- the input bench.py
  times.

ak.sum, ak.max and ak.argmax(axis=-1) run through the C ABI on the GPU and
are compared with the C oracle run over all host cores: argmax indices and
max values bit for bit, sums within 4*n*eps*sum|x| of the FP64
compensated-sum oracle, with the error figures printed.
"""

import os

import numpy as np
import pytest

import oracle
from bench import make_c1

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nlists", [1_000_000, 10_000_000])
def test_c1_reducers_against_the_oracle(nlists):
    import torch

    import awkward_gb300

    off, x = make_c1(nlists, 0)
    n = nlists
    be = awkward_gb300.backend()
    d_off, d_x = torch.from_numpy(off).cuda(), torch.from_numpy(x).cuda()
    g_sum = torch.empty(n, dtype=torch.float64, device="cuda")
    g_max = torch.empty(n, dtype=torch.float64, device="cuda")
    g_arg = torch.empty(n, dtype=torch.int64, device="cuda")
    be["awkward_reduce_sum", np.float64, np.float64, np.int64](g_sum, d_x, d_off, n)
    be["awkward_reduce_max", np.float64, np.float64, np.int64](g_max, d_x, d_off, n, -np.inf)
    be["awkward_reduce_argmax", np.int64, np.float64, np.int64, np.int64](
        g_arg, d_x, d_off, d_off[:-1].contiguous(), n)
    be.synchronize()
    threads = os.cpu_count() or 1
    e_max, e_arg = np.empty(n), np.empty(n, np.int64)
    oracle.parallel_reduce("awkward_reduce_max_float64_float64_64", e_max, x, off, n, threads,
                           identity=-np.inf)
    oracle.parallel_reduce("awkward_reduce_argmax_float64_64", e_arg, x, off, n, threads)
    np.testing.assert_array_equal(g_arg.cpu().numpy(), e_arg)
    np.testing.assert_array_equal(g_max.cpu().numpy().view(np.int64), e_max.view(np.int64))
    rep = oracle.sum_error_report(g_sum.cpu().numpy(), x, off, nthreads=threads)
    print(f"sum_err C1 {nlists} lists: {rep}")
    assert rep["nonfinite_ok"] and rep["within"], rep
