"""The single-colony autotuner (aco_colony_autotune): whatever kernel and
launch shape it keeps, the colony afterwards starts from its initialised
state and evolves bit for bit like the port."""
import os

import pytest

import oracle
import acogpu_gb300 as aco
from acogpu_gb300 import _abi
from helpers import assert_same_state, instance

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 4
MODES = {_abi.ACO_CONSTRUCT_STAGED, _abi.ACO_CONSTRUCT_CLUSTER, _abi.ACO_CONSTRUCT_DIRECT,
         _abi.ACO_CONSTRUCT_ROWS, _abi.ACO_CONSTRUCT_GLOBAL}


def _tuned_vs_port(d, p, iters, ctx):
    g = aco.Colony(d, params=p, num_ants=p.num_ants)
    g.initialize()
    t = g.autotune()
    assert t["construct_mode"] in MODES and t["construct_ms"] > 0, t
    q = oracle.Port(p, d, threads=THREADS)
    q.initialize()
    for it in range(iters):
        g.constructSolution()
        q.iterate()
        assert_same_state(g, q, aging=bool(p.aging), ctx=f"{ctx} ({t}) iteration {it}")
    g.close()
    q.close()
    return t


def test_autotuned_rank_based_with_aging():
    _, _, d = instance(1000, 81, kind="clustered")
    p = _abi.default_params(num_ants=1000, variant=_abi.ACO_RANK_BASED, rank_w=6, aging=1,
                            cand_k=30, rho=0.1, beta=2.0, nn_order=_abi.ACO_NN_STABLE,
                            heuristic=_abi.ACO_HEURISTIC_DEVICE, fallback=_abi.ACO_FALLBACK_BEST,
                            tau0_mode=_abi.ACO_TAU0_DORIGO, seed=81)
    _tuned_vs_port(d, p, 4, "RBAS k=30")


def test_autotuned_ant_system_two_tables():
    """n = 1500, k = 20: the staged table fits, the cluster and direct
    kernels are candidates too, with several ants per CTA."""
    _, _, d = instance(1500, 82)
    p = _abi.default_params(num_ants=600, cand_k=20, rho=0.2, beta=2.0,
                            nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO,
                            seed=82)
    _tuned_vs_port(d, p, 3, "AS k=20")


def test_autotuned_full_rows():
    _, _, d = instance(400, 83, kind="clustered")
    p = _abi.default_params(num_ants=200, aging=1, cand_k=0, rho=0.1, beta=2.0, seed=83)
    t = _tuned_vs_port(d, p, 3, "full rows")
    assert t["construct_mode"] in (_abi.ACO_CONSTRUCT_ROWS, _abi.ACO_CONSTRUCT_GLOBAL)
