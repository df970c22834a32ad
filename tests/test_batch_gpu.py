"""GPU tests of batches of uneven instances (one persistent construction
launch over a per-instance work queue, graph-replayed iterations): every
instance must evolve exactly like a colony created on its own."""
import numpy as np
import pytest

import acogpu_gb300 as aco
from acogpu_gb300 import _abi, instances
from helpers import is_permutation_rows, tour_lengths

pytestmark = pytest.mark.gpu
GOLDEN_STEP = np.uint64(0x9E3779B97F4A7C15)


def make_instances(sizes, seed):
    out = []
    for i, n in enumerate(sizes):
        gen = instances.uniform_instance if i % 2 == 0 else instances.clustered_instance
        out.append(gen(int(n), seed=seed + i))
    return out


def fast_params(**kw):
    base = dict(nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO, cand_k=20,
                beta=2.0, rho=0.1, seed=777)
    base.update(kw)
    return _abi.default_params(**base)


def single(inst, p, i, cap):
    q = _abi.AcoParams.from_buffer_copy(p)
    n = len(inst[0])
    q.num_ants = min(cap, n)
    with np.errstate(over="ignore"):
        q.seed = int(np.uint64(p.seed) + np.uint64(i) * GOLDEN_STEP)
    c = aco.Colony(coords=inst, params=q, num_ants=q.num_ants)
    c.initialize()
    return c


@pytest.mark.parametrize("variant,aging", [(_abi.ACO_ANT_SYSTEM, 0), (_abi.ACO_RANK_BASED, 1)])
@pytest.mark.parametrize("tune", [False, True])
@pytest.mark.parametrize("mode", [_abi.ACO_CONSTRUCT_AUTO, _abi.ACO_CONSTRUCT_GLOBAL],
                         ids=["staged", "l2rows"])
def test_batch_instances_match_single_colonies(variant, aging, tune, mode):
    """Staged items (tables in shared memory) and L2-row items in one launch:
    the 2000-city table (k = 20: 240 KB) does not fit in shared memory."""
    sizes = [57, 120, 2000, 333, 64, 1300, 95]
    insts = make_instances(sizes, 300)
    p = fast_params(variant=variant, rank_w=6, aging=aging, construct_mode=mode)
    if aging:
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (3, 6, 2, 20)
    cap = 80
    b = aco.Batch(insts, params=p, num_ants=cap)
    b.initialize()
    if tune:
        t = b.autotune()
        assert t["ants_per_block"] in (1, 2, 4, 8, 16, 20) and t["row_threads"] in (128, 256, 512)
        assert t["staged_instances"] == (0 if mode == _abi.ACO_CONSTRUCT_GLOBAL else len(sizes) - 1)
    iters = 8
    b.run(iters)
    b.synchronize()
    best = b.glob_best()
    for i, inst in enumerate(insts):
        c = single(inst, p, i, cap)
        for _ in range(iters):
            c.constructSolution()
        v = b.colony(i)
        assert np.array_equal(v.tours(), c.tours()), f"instance {i}: tours"
        assert np.array_equal(v.tour_lengths(), c.tour_lengths()), f"instance {i}: lengths"
        assert np.array_equal(v.pheromone().view(np.uint32), c.pheromone().view(np.uint32)), i
        assert best[i] == c.getGlobBestDist()
        if aging:
            a, s = v.aging_state(), c.aging_state()
            assert np.array_equal(a["age"], s["age"]) and np.array_equal(a["valid"], s["valid"])
        c.close()
    assert b.tours_built() > 0
    b.close()


def test_uneven_batch_properties():
    """Sizes log-uniform in [50, 2000], uniform/clustered alternating, ants
    capped at 1024, k = 20: valid tours and lengths after a few iterations."""
    sizes = instances.batch_sizes(24, seed=11)
    sizes[0], sizes[1] = 2000, 50
    insts = make_instances(sizes, 900)
    b = aco.Batch(insts, params=fast_params(), num_ants=1024)
    b.initialize()
    b.autotune()
    before = b.glob_best()
    launches0 = b.launch_count()
    b.run(3)
    b.synchronize()
    after = b.glob_best()
    assert np.all(after <= before)
    for i in (0, 1, 5, 17):
        v = b.colony(i)
        n = sizes[i]
        t = v.tours()
        d = instances.euc2d_distances(*insts[i])
        assert is_permutation_rows(t, n)
        assert np.array_equal(tour_lengths(d, t), v.tour_lengths())
    assert b.launch_count() - launches0 == 9  # three launches per batch iteration
    built = b.tours_built()
    b.run(2)  # graph replays only: the state read after them must be fresh
    b.synchronize()
    assert b.tours_built() - built == 2 * sum(min(n, 1024) for n in sizes)
    assert np.all(b.glob_best() <= after)
    b.close()


def test_coincident_cities_batch_matches_general_kernel():
    """Instances with coincident triples (infinite candidate weights at
    positions 0 and 1, +inf weight sums) in one batch: the staged and L2-row
    items reproduce single colonies on the general kernel, whose ordered fold
    needs no masked products."""
    insts = []
    for i, n in enumerate([300, 1500, 90]):
        x, y = instances.uniform_instance(n, seed=40 + i)
        x, y = np.array(x), np.array(y)
        pick = np.random.default_rng(40 + i).choice(n, 3 * (n // 30), replace=False)
        for a, b2, c2 in pick.reshape(-1, 3):
            x[b2] = x[c2] = x[a]
            y[b2] = y[c2] = y[a]
        insts.append((x, y))
    p = fast_params()
    cap = 64
    b = aco.Batch(insts, params=p, num_ants=cap)
    b.initialize()
    b.run(4)
    b.synchronize()
    g = _abi.AcoParams.from_buffer_copy(p)
    g.construct_mode = _abi.ACO_CONSTRUCT_GLOBAL
    for i, inst in enumerate(insts):
        c = single(inst, g, i, cap)
        for _ in range(4):
            c.constructSolution()
        v = b.colony(i)
        assert np.array_equal(v.tours(), c.tours()), f"instance {i}: tours"
        assert np.array_equal(v.pheromone().view(np.uint32), c.pheromone().view(np.uint32)), i
        c.close()
    b.close()


@pytest.mark.parametrize("apb", [16, 20])
def test_batch_with_many_ants_per_cta(apb):
    """The largest ants-per-CTA shapes of the batch kernel (20 warps fit its
    register budget) build the same tours as single colonies."""
    sizes = [900, 57, 1500, 333]
    insts = make_instances(sizes, 301)
    p = fast_params()
    b = aco.Batch(insts, params=p, num_ants=300)
    b.initialize()
    b.set_tuning(apb, 0)
    b.run(4)
    b.synchronize()
    for i, inst in enumerate(insts):
        c = single(inst, p, i, 300)
        for _ in range(4):
            c.constructSolution()
        v = b.colony(i)
        assert np.array_equal(v.tours(), c.tours()), f"apb {apb} instance {i}: tours"
        assert np.array_equal(v.pheromone().view(np.uint32), c.pheromone().view(np.uint32)), i
        c.close()
    b.close()
