"""A seeded sweep of the oracle against the reference's own compiled CPU path
(where its sources are present): random small instances (uniform or
clustered, some with coincident cities), both nn tie orders, noaging and
aging builds, several beta and rho; full rows, the reference's only
construction rule.  Every iteration's tours, lengths, pheromone bits and
bests must agree."""
import numpy as np
import pytest

import oracle
from acogpu_gb300 import _abi, instances
from helpers import bits, params

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="reference sources absent")


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_compiled_reference_sweep(seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(8, 90))
    gen = instances.uniform_instance if rng.random() < 0.5 else instances.clustered_instance
    x, y = gen(n, seed=int(rng.integers(1 << 30)))
    x, y = np.array(x), np.array(y)
    if rng.random() < 0.3:
        for a, b, c in rng.choice(n, 3 * max(1, n // 20), replace=False).reshape(-1, 3):
            x[b] = x[c] = x[a]
            y[b] = y[c] = y[a]
    d = instances.euc2d_distances(x, y)
    m = int(rng.integers(2, 60))
    aging = int(rng.random() < 0.5)
    stable = bool(rng.random() < 0.5)
    p = params(num_ants=m, beta=float(rng.choice([1.0, 2.0, 5.0])),
               rho=float(rng.choice([0.1, 0.2, 0.5])), aging=aging,
               seed=int(rng.integers(1 << 30)),
               nn_order=_abi.ACO_NN_STABLE if stable else _abi.ACO_NN_REFERENCE_QSORT)
    if aging:
        mr = int(rng.integers(2, 6))
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (mr, mr + int(rng.integers(1, 4)), 2, max(1, m // 2))
    ref = oracle.Ref(p, d, stable_nn=stable)
    ref.initialize()
    q = oracle.Port(p, d, threads=2)
    q.initialize()
    ctx = f"seed {seed}: n{n} m{m} aging{aging} stable{stable} beta{p.beta} rho{p.rho}"
    assert np.array_equal(ref.nn(), q.nn()), ctx
    for it in range(int(rng.integers(3, 12))):
        ref.iterate()
        q.iterate()
        assert np.array_equal(ref.tours(), q.tours()), (ctx, it)
        assert np.array_equal(ref.lengths(), q.lengths()), (ctx, it)
        assert np.array_equal(bits(ref.pheromone()), bits(q.pheromone())), (ctx, it)
        assert (ref.iter_best(), ref.glob_best()) == (q.iter_best(), q.glob_best()), (ctx, it)
        if aging:
            a, b = ref.aging_state(), q.aging()
            for key in ("age", "perf", "valid"):
                assert np.array_equal(a[key], b[key]), (ctx, it, key)
    ref.close()
    q.close()
