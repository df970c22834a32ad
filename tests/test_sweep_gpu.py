"""A seeded sweep over the configuration space against the oracle: sizes
from 5 to 3200 cities, candidate lists from 1 to the full row, both
variants, aging, every construction mode, the fallback tier on and off, both
nn tie orders, coincident cities.  Each case runs a few iterations and must
stay bit-identical; the cases are fixed by the seed."""
import numpy as np
import pytest

import oracle
import acogpu_gb300 as aco
from acogpu_gb300 import _abi, instances
from helpers import assert_same_state

pytestmark = pytest.mark.gpu


def case(rng):
    n = int(rng.choice([rng.integers(5, 60), rng.integers(60, 1200), rng.integers(1200, 3200)]))
    gen = instances.clustered_instance if rng.random() < 0.5 else instances.uniform_instance
    x, y = gen(n, seed=int(rng.integers(1 << 30)))
    x, y = np.array(x), np.array(y)
    if rng.random() < 0.3:  # coincident triples: distance 0, infinite weights
        for a, b, c in rng.choice(n, 3 * max(1, n // 40), replace=False).reshape(-1, 3):
            x[b] = x[c] = x[a]
            y[b] = y[c] = y[a]
    m = int(rng.integers(1, 200))
    k = int(rng.choice([1, 3, 8, 16, 20, 24, 30, 32, 40, 0]))
    if k == 0 and n > 300:
        k = 32  # the oracle's full-row roulette is O(m n^2) per iteration
    full = k == 0 or k >= n
    modes = [_abi.ACO_CONSTRUCT_AUTO, _abi.ACO_CONSTRUCT_GLOBAL]
    if 0 < k <= 32 and n > 2048:
        modes += [_abi.ACO_CONSTRUCT_DIRECT, _abi.ACO_CONSTRUCT_CLUSTER]
    aging = int(rng.random() < 0.4)
    p = _abi.default_params(
        num_ants=m, cand_k=k, beta=float(rng.choice([1.0, 2.0, 5.0])),
        rho=float(rng.choice([0.1, 0.5])), seed=int(rng.integers(1 << 30)),
        variant=int(rng.choice([_abi.ACO_ANT_SYSTEM, _abi.ACO_RANK_BASED])),
        rank_w=int(rng.integers(2, 8)), aging=aging, construct_mode=int(rng.choice(modes)),
        fallback_tier=int(rng.choice([0, 1, 2])),
        nn_order=int(rng.choice([_abi.ACO_NN_STABLE, _abi.ACO_NN_REFERENCE_QSORT])),
        heuristic=_abi.ACO_HEURISTIC_DEVICE,
        fallback=_abi.ACO_FALLBACK_REFERENCE if full else _abi.ACO_FALLBACK_BEST,
        tau0_mode=_abi.ACO_TAU0_DORIGO)
    if aging:
        mr = int(rng.integers(2, 8))
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (mr, mr + int(rng.integers(1, 5)), 2, max(1, m // 2))
    return p, instances.euc2d_distances(x, y), int(rng.integers(2, 7))


@pytest.mark.parametrize("seed", [101, 202, 303])
def test_seeded_sweep_matches_oracle(seed):
    rng = np.random.default_rng(seed)
    for i in range(25):
        p, d, iters = case(rng)
        ctx = (f"seed {seed} case {i}: n{d.shape[0]} m{p.num_ants} k{p.cand_k} "
               f"variant{p.variant} aging{p.aging} mode{p.construct_mode} "
               f"tier{p.fallback_tier} nn{p.nn_order}")
        g = None
        try:
            g = aco.Colony(d, params=p, num_ants=p.num_ants)
            g.initialize()
        except aco.AcoError as e:  # a forced mode this device cannot run
            assert e.status == _abi.ACO_ERR_UNSUPPORTED, ctx
            if g is not None:
                g.close()
            continue
        q = oracle.Port(p, d, threads=8)
        q.initialize()
        for it in range(iters):
            g.constructSolution()
            q.iterate()
            assert_same_state(g, q, aging=bool(p.aging), ctx=f"{ctx} iteration {it}")
        g.close()
        q.close()
