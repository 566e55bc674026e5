"""Kernel-table argument checks that fail before any CUDA call (run without a GPU):
a pointer argument, or a row of a list-of-lists argument, that is not a CUDA
tensor raises TypeError naming the specialization and the argument."""

import numpy as np
import pytest
import torch

import awkward_gb300


def test_pointer_argument_must_be_a_cuda_tensor():
    k = awkward_gb300.backend()["awkward_reduce_sum", np.float64, np.float64, np.int64]
    with pytest.raises(TypeError, match="awkward_reduce_sum_float64_float64_64: argument toptr"):
        k(torch.zeros(3, dtype=torch.float64), torch.zeros(3, dtype=torch.float64),
          torch.zeros(4, dtype=torch.int64), 3)


def test_rows_of_a_list_argument_must_be_cuda_tensors():
    k = awkward_gb300.backend().by_name("awkward_ListArray64_combinations_64")
    rows = [torch.zeros(4, dtype=torch.int64) for _ in range(2)]
    with pytest.raises(TypeError, match="rows of tocarry"):
        k(rows, torch.zeros(2, dtype=torch.int64), torch.zeros(2, dtype=torch.int64), 2, False,
          torch.zeros(2, dtype=torch.int64), torch.zeros(2, dtype=torch.int64), 2)
