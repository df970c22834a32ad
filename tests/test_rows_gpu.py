"""GPU parity of the long-row construction kernel (k > 32, full rows
included; k_construct_rows.cu) against the port: its two modes of the same
colony, rows longer than one scan round (n > 1024), candidate lists of
64 and 100 with the best-choice fallback, coincident cities (infinite
weights), ants that blend their fitness after convergence, and batches whose
instances differ in size."""
import os

import numpy as np
import pytest

import oracle
import acogpu_gb300 as aco
from acogpu_gb300 import _abi, instances
from helpers import assert_same_state, bits, instance

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 4
GOLDEN_STEP = np.uint64(0x9E3779B97F4A7C15)


def run_vs_port(d, p, iters, ctx, mode=_abi.ACO_CONSTRUCT_AUTO):
    q_ = _abi.AcoParams.from_buffer_copy(p)
    q_.construct_mode = mode
    g = aco.Colony(d, params=q_, num_ants=p.num_ants)
    g.initialize()
    q = oracle.Port(p, d, threads=THREADS)
    q.initialize()
    for it in range(iters):
        g.constructSolution()
        q.iterate()
        assert_same_state(g, q, aging=bool(p.aging), ctx=f"{ctx} iteration {it}")
    g.close()
    q.close()


@pytest.mark.parametrize("mode", [_abi.ACO_CONSTRUCT_ROWS, _abi.ACO_CONSTRUCT_GLOBAL])
def test_rows_and_general_kernels_agree_with_the_port(mode):
    _, _, d = instance(700, 71, kind="clustered")
    p = _abi.default_params(num_ants=300, aging=1, cand_k=0, rho=0.1, beta=2.0, seed=71)
    run_vs_port(d, p, 4, f"mode {mode}", mode)


def test_rows_longer_than_one_scan_round():
    """n = 2000: two rounds of 1024 row entries per scan, and the guess taken
    from the compacted buffer."""
    _, _, d = instance(2000, 72)
    p = _abi.default_params(num_ants=160, cand_k=0, rho=0.1, beta=2.0, seed=72)
    run_vs_port(d, p, 3, "n=2000")


@pytest.mark.parametrize("k,variant", [(64, _abi.ACO_ANT_SYSTEM), (100, _abi.ACO_RANK_BASED)])
def test_candidate_lists_longer_than_32(k, variant):
    _, _, d = instance(600, 73 + k, kind="clustered")
    p = _abi.default_params(num_ants=200, variant=variant, rank_w=6, cand_k=k, rho=0.2,
                            beta=2.0, nn_order=_abi.ACO_NN_STABLE,
                            heuristic=_abi.ACO_HEURISTIC_DEVICE, fallback=_abi.ACO_FALLBACK_BEST,
                            tau0_mode=_abi.ACO_TAU0_DORIGO, seed=73 + k)
    run_vs_port(d, p, 5, f"k={k}")


def test_coincident_cities_full_rows():
    """Cities at distance 0 give infinite weights: +inf sums and the walk
    past the row into select_local_best, as the reference does."""
    x, y = instances.uniform_instance(120, seed=74)
    x = np.asarray(x, np.float32).copy()
    y = np.asarray(y, np.float32).copy()
    for a, b in ((3, 40), (7, 41), (90, 91)):
        x[b], y[b] = x[a], y[a]
    d = instances.euc2d_distances(x, y)
    p = _abi.default_params(num_ants=60, cand_k=0, rho=0.3, beta=2.0, seed=74)
    run_vs_port(d, p, 6, "coincident")


def test_blending_ants_after_convergence():
    """Small aging limits so the colony converges early: recruits blend
    their fitness (tau and eta read from L2) for min_ret iterations."""
    _, _, d = instance(220, 75, kind="clustered")
    p = _abi.default_params(num_ants=90, aging=1, cand_k=0, rho=0.2, beta=2.0, seed=75)
    (p.min_retirement_age, p.max_retirement_age, p.local_performance, p.global_performance,
     p.min_population_limit, p.max_population_limit) = (4, 7, 10, 2, 20, 100)
    g = aco.Colony(d, params=p, num_ants=90)
    g.initialize()
    q = oracle.Port(p, d, threads=THREADS)
    q.initialize()
    blended = False
    for it in range(45):
        g.constructSolution()
        q.iterate()
        a = q.aging()
        blended = blended or (a["isconverged"] and bool(((a["age"] < 4) & (a["valid"] > 0)).any()))
        assert_same_state(g, q, aging=True, ctx=f"iteration {it}")
    assert blended
    g.close()
    q.close()


def test_batch_of_long_rows_of_uneven_size():
    """One launch over instances of 300, 1500 and 2000 cities (full rows,
    aging): the per-ant regions are sized for the largest; every instance
    against its own port."""
    insts = [instances.clustered_instance(n, seed=76 + i) for i, n in enumerate((300, 1500, 2000))]
    p = _abi.default_params(num_ants=120, aging=1, cand_k=0, rho=0.1, beta=2.0, seed=76)
    b = aco.Batch(insts, params=p, num_ants=120)
    b.initialize()
    ports = []
    for i, (x, y) in enumerate(insts):
        qi = _abi.AcoParams.from_buffer_copy(p)
        with np.errstate(over="ignore"):
            qi.seed = int(np.uint64(p.seed) + np.uint64(i) * GOLDEN_STEP)
        q = oracle.Port(qi, instances.euc2d_distances(x, y), threads=THREADS)
        q.initialize()
        ports.append(q)
    for it in range(3):
        b.run(1)
        b.synchronize()
        for i, q in enumerate(ports):
            q.iterate()
            assert_same_state(b.colony(i), q, aging=True, ctx=f"instance {i} iteration {it}")
    t = b.autotune()
    assert t["ants_per_block"] in (2, 4, 6, 8, 11)
    for q in ports:
        q.close()
    b.close()
