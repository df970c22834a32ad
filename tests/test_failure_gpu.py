"""Failure paths on the GPU without a fault: a bounded device wait that runs
out (the kernel records the timeout and returns; the context stays usable),
and device allocation failures injected on the host (creation fails with
ACO_ERR_OUT_OF_MEMORY, nothing leaks, the next creation works)."""
import numpy as np
import pytest

import acogpu_gb300 as aco
from acogpu_gb300 import _abi
from acogpu_gb300.colony import AcoError, lib
from helpers import instance, params

pytestmark = pytest.mark.gpu

FAST = dict(nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO)


def small_colony(seed=3):
    _, _, d = instance(80, seed)
    p = params(num_ants=16, beta=2.0, rho=0.2, cand_k=10, seed=seed, **FAST)
    return aco.Colony(d, params=p, num_ants=16)


def run_twice_same(seed=3):
    bests = []
    for _ in range(2):
        c = small_colony(seed)
        c.initialize()
        for _ in range(3):
            c.constructSolution()
        bests.append((c.getGlobBestDist(), c.tours().copy()))
        c.close()
    return bests


def test_bounded_wait_times_out_and_the_context_survives():
    L = lib()
    assert L.aco_selftest_bounded_wait(1 << 12) == _abi.ACO_ERR_DEVICE_TIMEOUT
    assert L.aco_selftest_bounded_wait(0) == _abi.ACO_ERR_INVALID_ARGUMENT
    (b0, t0), (b1, t1) = run_twice_same()
    assert b0 == b1 and b0 > 0 and np.array_equal(t0, t1)


@pytest.mark.parametrize("after", [0, 1, 4, 9, 16, 24])
def test_injected_allocation_failure_is_clean(after):
    import torch
    L = lib()
    small_colony().close()  # first-use allocations of the runtime happen here
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    L.aco_debug_fail_allocation(after)
    try:
        with pytest.raises(AcoError) as err:
            small_colony()
        assert err.value.status == _abi.ACO_ERR_OUT_OF_MEMORY
    finally:
        L.aco_debug_fail_allocation(-1)
    torch.cuda.synchronize()
    assert abs(torch.cuda.mem_get_info()[0] - free0) < (4 << 20)  # nothing left behind
    (b0, t0), (b1, t1) = run_twice_same()
    assert b0 == b1 and np.array_equal(t0, t1)
