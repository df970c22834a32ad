"""GPU test of aco_nn_list_reference_order_noalloc, the nn-list entry point
that allocates no device memory (for callers that cannot call cudaMalloc or
cudaFree).  Its rows must equal those the colony path builds with its
allocated scratch.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import acogpu_gb300 as aco
from acogpu_gb300 import _abi
from helpers import instance, params

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    L = aco.lib()
    f = L.aco_nn_list_reference_order_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _colony_rows(d):
    """Rows built by the existing entry points (colony with full-row
    candidates in the reference quicksort order)."""
    n = d.shape[0]
    col = aco.Colony(d, params=params(num_ants=4, nn_order=_abi.ACO_NN_REFERENCE_QSORT,
                                      heuristic=_abi.ACO_HEURISTIC_DEVICE), num_ants=4)
    col.initialize()
    rows = col.nn_list()
    col.close()
    assert rows.shape == (n, n)
    return rows


@pytest.mark.parametrize("n,seed", [(300, 41), (1024, 42)])
def test_noalloc_nn_list_matches_colony_path(n, seed):
    import torch
    f = _noalloc_fn()
    _, _, d = instance(n, seed, kind="clustered")
    expected = _colony_rows(d)
    dist = torch.from_numpy(d).cuda()
    out = torch.full((n, n), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row share the static scratch
        out.fill_(-7)
        torch.cuda.synchronize()
        st = f(dist.data_ptr(), n, out.data_ptr(), stream)
        assert st == _abi.ACO_OK, f"call {call}: status {st}"
        assert np.array_equal(out.cpu().numpy(), expected), f"call {call}: rows differ"


def test_noalloc_rejects_sizes_above_the_limit():
    import torch
    f = _noalloc_fn()
    n = 1025
    dist = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    out = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    assert f(dist.data_ptr(), n, out.data_ptr(), None) == _abi.ACO_ERR_UNSUPPORTED
    assert f(None, 10, out.data_ptr(), None) == _abi.ACO_ERR_INVALID_ARGUMENT
