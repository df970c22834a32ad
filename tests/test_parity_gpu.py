"""GPU parity: the CUDA path against the CPU oracle (bit-exact) and against
the golden fixtures recorded from the reference's own CPU path."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
import acogpu_gb300 as aco
from acogpu_gb300 import _abi
from helpers import assert_same_state, bits, instance, is_permutation_rows, params, tour_lengths

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = json.load(open(os.path.join(GOLDEN, "cases.json")))


def pair(p, d, threads=8):
    g = aco.Colony(d, params=p, num_ants=p.num_ants)
    g.initialize()
    q = oracle.Port(p, d, threads=threads)
    q.initialize()
    return g, q


def run_pair(p, d, iters, use_graph=False, ctx=""):
    g, q = pair(p, d)
    assert np.array_equal(g.nn_list(), q.nn()), f"{ctx}: nn-list"
    assert np.array_equal(bits(g.heuristic()), bits(q.heuristic())), f"{ctx}: heuristic"
    assert np.array_equal(bits(g.pheromone()), bits(q.pheromone())), f"{ctx}: tau0"
    assert np.array_equal(bits(g.choice_info()), bits(q.choice())), f"{ctx}: choice-info"
    for it in range(iters):
        if use_graph:
            g.run(1)
        else:
            g.constructSolution()
        q.iterate()
        assert_same_state(g, q, aging=bool(p.aging), ctx=f"{ctx} iteration {it}")
    g.close()
    q.close()


# ---------------------------------------------------------------- golden
def golden_params(meta):
    p = params(num_ants=meta["m"], beta=meta["beta"], rho=meta["rho"], aging=meta["aging"],
               seed=meta["seed_stream"],
               nn_order=_abi.ACO_NN_STABLE if meta["stable"] else _abi.ACO_NN_REFERENCE_QSORT)
    if meta["aging"]:
        (p.min_retirement_age, p.max_retirement_age, p.local_performance, p.global_performance,
         p.min_population_limit, p.max_population_limit) = meta["six"]
    return p


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference_golden(name):
    """Reference parity mode (full-row candidates, reference quicksort order,
    libm heuristic, reference fallback, deterministic deposit, tau0 = 1e-6):
    every iteration's tours, integer lengths and bests, and the pheromone
    matrix, equal the reference's own CPU run."""
    meta = CASES[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    col = aco.Colony(coords=(g["x"], g["y"]), params=golden_params(meta), num_ants=meta["m"])
    assert np.array_equal(col.distances(), g["dist"])
    col.initialize()
    assert np.array_equal(col.nn_list(), g["nn"])
    assert np.array_equal(bits(col.heuristic()), bits(g["eta"]))
    for it in range(meta["iters"]):
        col.constructSolution()
        assert np.array_equal(col.tours(), g["tours"][it]), f"iteration {it}: tours"
        assert np.array_equal(col.tour_lengths(), g["lengths"][it]), f"iteration {it}: lengths"
        assert col.getIterBestDist() == g["iter_best"][it]
        assert col.getGlobBestDist() == g["glob_best"][it]
        assert col.getNumValidAnts() == g["num_valid"][it]
        h = hashlib.sha256(col.pheromone().tobytes()).hexdigest()
        assert h == meta["tau_hashes"][it], f"iteration {it}: pheromone"
    assert np.array_equal(col.best_tour(), g["best_tour"])
    col.close()


# ---------------------------------------------------------------- oracle
REFERENCE_MODE = dict(nn_order=_abi.ACO_NN_REFERENCE_QSORT, heuristic=_abi.ACO_HEURISTIC_LIBM,
                      fallback=_abi.ACO_FALLBACK_REFERENCE)
FAST_MODE = dict(nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                 fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO)


@pytest.mark.parametrize("case", [
    dict(n=24, m=16, beta=2.0, rho=0.5, iters=10, **REFERENCE_MODE),
    dict(n=31, m=20, beta=2.0, rho=0.3, iters=20, aging=1, six=(3, 5, 10, 2, 10, 100),
         **REFERENCE_MODE),
    dict(n=60, m=40, beta=2.0, rho=0.5, iters=8, **REFERENCE_MODE),
    dict(n=97, m=33, beta=5.0, rho=0.1, iters=6, kind="clustered", **REFERENCE_MODE),
    dict(n=50, m=30, beta=2.0, rho=0.3, iters=30, aging=1, six=(3, 5, 10, 2, 15, 100),
         **REFERENCE_MODE),
    dict(n=80, m=50, beta=2.0, rho=0.2, iters=10, cand_k=16, **FAST_MODE),
    dict(n=90, m=40, beta=3.0, rho=0.2, iters=25, cand_k=20, aging=1, six=(3, 6, 10, 2, 20, 100),
         **FAST_MODE),
    dict(n=130, m=64, beta=2.0, rho=0.1, iters=10, cand_k=40, **FAST_MODE),
    dict(n=120, m=60, beta=2.0, rho=0.1, iters=15, cand_k=30, variant=_abi.ACO_RANK_BASED,
         rank_w=6, aging=1, six=(3, 6, 10, 2, 30, 100), kind="clustered", **FAST_MODE),
    dict(n=70, m=35, beta=2.0, rho=0.3, iters=8, variant=_abi.ACO_RANK_BASED, rank_w=5,
         **REFERENCE_MODE),
    dict(n=64, m=20, beta=2.0, rho=0.5, iters=8, cand_k=0, nn_order=_abi.ACO_NN_STABLE,
         heuristic=_abi.ACO_HEURISTIC_DEVICE, fallback=_abi.ACO_FALLBACK_BEST),
], ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items() if k not in ("six",)))
def test_gpu_matches_oracle(case):
    case = dict(case)
    case["num_ants"] = case.pop("m")
    n, seed = case.pop("n"), 100 + case["num_ants"]
    iters = case.pop("iters")
    kind = case.pop("kind", "uniform")
    six = case.pop("six", None)
    _, _, d = instance(n, seed, kind=kind)
    p = params(seed=seed, **case)
    if six:
        (p.min_retirement_age, p.max_retirement_age, p.local_performance, p.global_performance,
         p.min_population_limit, p.max_population_limit) = six
    run_pair(p, d, iters, ctx=str(case))


def test_graph_replay_matches_oracle():
    _, _, d = instance(75, 3)
    p = params(num_ants=30, beta=2.0, rho=0.2, cand_k=24, seed=9, **FAST_MODE)
    run_pair(p, d, 6, use_graph=True, ctx="graph")


@pytest.mark.parametrize("mode", [_abi.ACO_CONSTRUCT_GLOBAL, _abi.ACO_CONSTRUCT_STAGED])
@pytest.mark.parametrize("aging", [0, 1])
def test_construct_kernels_match_oracle(mode, aging):
    """The shared-memory-staged and the global-memory construction kernels
    both reproduce the oracle."""
    _, _, d = instance(150, 6, kind="clustered")
    p = params(num_ants=70, beta=2.0, rho=0.2, cand_k=30, seed=6, construct_mode=mode,
               aging=aging, **FAST_MODE)
    if aging:
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (3, 6, 2, 35)
    run_pair(p, d, 12 if aging else 5, ctx=f"mode{mode}")


@pytest.mark.parametrize("m,six,iters", [
    (120, (10, 12, 2, 100), 40),   # after convergence up to 10 blend ants per iteration
    (400, (300, 5, 2, 390), 12),   # more blend ants than SMs: blend CTAs restage the table
])
def test_staged_blend_ants_match_oracle(m, six, iters):
    """Aging colonies on the staged kernel: ants that blend run on a table of
    their own blended weights (one CTA each), the others on the plain table;
    tours, lengths, pheromone and ages stay bit-identical to the oracle."""
    _, _, d = instance(200, 77, kind="clustered")
    p = params(num_ants=m, beta=2.0, rho=0.2, cand_k=20, seed=77, aging=1,
               construct_mode=_abi.ACO_CONSTRUCT_STAGED, **FAST_MODE)
    (p.min_retirement_age, p.max_retirement_age, p.global_performance,
     p.min_population_limit) = six
    run_pair(p, d, iters, ctx=f"blend m{m}")


@pytest.mark.parametrize("mode", ["direct", "cluster"])
@pytest.mark.parametrize("n,k,aging", [(700, 24, 1), (1500, 32, 0), (3000, 20, 1),
                                       (5000, 32, 0), (8192, 16, 0)])
def test_large_table_kernels_match_oracle(n, k, aging, mode):
    """k <= 32 with a candidate table too large for one CTA's shared memory:
    the step loop on rows read from L2 (direct) or on the table split over a
    cluster of ceil(n/1024) CTAs read through distributed shared memory
    (cluster: 1, 2, 3, 5 and 8 CTAs), with the tabu list in 2, 2, 4, 8 and 8
    registers per lane, reproduces the oracle (aging: through the blend and
    its fallback)."""
    _, _, d = instance(n, 50 + n, kind="clustered")
    cm = _abi.ACO_CONSTRUCT_DIRECT if mode == "direct" else _abi.ACO_CONSTRUCT_CLUSTER
    p = params(num_ants=24, beta=2.0, rho=0.2, cand_k=k, seed=n, aging=aging,
               construct_mode=cm, **FAST_MODE)
    if aging:
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (3, 6, 2, 20)
    run_pair(p, d, 10 if aging else 3, ctx=f"{mode} n{n}")


def coincident_instance(n, seed, groups):
    """Uniform cities with `groups` triples of them moved onto one point:
    distance 0, infinite heuristic weights at candidate positions 0 and 1 of
    their rows, and sums of candidate weights that are +inf."""
    from acogpu_gb300 import instances
    x, y = instances.uniform_instance(n, box=10000, seed=seed)
    x, y = np.array(x), np.array(y)
    pick = np.random.default_rng(seed).choice(n, 3 * groups, replace=False).reshape(groups, 3)
    for a, b, c in pick:
        x[b] = x[c] = x[a]
        y[b] = y[c] = y[a]
    return instances.euc2d_distances(x, y)


@pytest.mark.parametrize("mode", [_abi.ACO_CONSTRUCT_GLOBAL, _abi.ACO_CONSTRUCT_STAGED,
                                  _abi.ACO_CONSTRUCT_DIRECT, _abi.ACO_CONSTRUCT_CLUSTER])
def test_coincident_cities_match_oracle(mode):
    """Infinite candidate weights anywhere in a row (not only first): the
    reference's walk then ends at candidate 0 (u*S NaN) or in the fallback,
    and every construction kernel takes the same branch."""
    d = coincident_instance(1100, 31, 40)
    assert (d[~np.eye(1100, dtype=bool)] == 0).any()
    p = params(num_ants=96, beta=2.0, rho=0.2, cand_k=20, seed=31, construct_mode=mode,
               **FAST_MODE)
    run_pair(p, d, 3, ctx=f"coincident mode{mode}")


@pytest.mark.parametrize("tier", [_abi.ACO_FALLBACK_TIER_ON, _abi.ACO_FALLBACK_TIER_OFF])
@pytest.mark.parametrize("n,mode,variant,aging", [
    (600, _abi.ACO_CONSTRUCT_STAGED, _abi.ACO_ANT_SYSTEM, 0),
    (600, _abi.ACO_CONSTRUCT_STAGED, _abi.ACO_RANK_BASED, 1),
    (2500, _abi.ACO_CONSTRUCT_CLUSTER, _abi.ACO_RANK_BASED, 0),
])
def test_fallback_tier_matches_oracle(tier, n, mode, variant, aging):
    """The best-choice fallback with its second tier (the next 128 neighbours
    and the row's largest choice value outside them) forced on or off, with
    8 candidates so that many steps fall back: the same tours as the
    oracle's scan of the whole row, through convergence."""
    _, _, d = instance(n, 17 + n, kind="clustered")
    p = params(num_ants=64, beta=2.0, rho=0.2, cand_k=8, seed=17, variant=variant, rank_w=6,
               aging=aging, construct_mode=mode, fallback_tier=tier, **FAST_MODE)
    if aging:
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (3, 6, 2, 40)
    run_pair(p, d, 25 if n <= 1000 else 6, ctx=f"tier{tier} n{n}")


@pytest.mark.parametrize("n,k", [(45, 16), (31, 30), (160, 30), (700, 1)])
def test_fallback_tier_edges_match_oracle(n, k):
    """The second tier at its edges: shorter than 128 neighbours (n = 45,
    k = 16: 28; n = 160), empty (n = 31, k = 30), and a single candidate
    (every step but one falls back)."""
    _, _, d = instance(n, 5 + n, kind="clustered")
    p = params(num_ants=48, beta=2.0, rho=0.2, cand_k=k, seed=5 + n,
               fallback_tier=_abi.ACO_FALLBACK_TIER_ON, **FAST_MODE)
    run_pair(p, d, 8, ctx=f"tier edges n{n} k{k}")


@pytest.mark.parametrize("n", [8, 22, 31])
@pytest.mark.parametrize("order", [_abi.ACO_NN_REFERENCE_QSORT, _abi.ACO_NN_STABLE])
def test_small_full_rows_match_oracle(n, order):
    """Full rows of at most 32 cities (k = n) on the staged kernel, with the
    reference fallback (the last unvisited city of the row): the rows' padding
    past n must never be taken for a city (a defect found by a randomized
    sweep: the reference-order sort left it unset)."""
    _, _, d = instance(n, 300 + n)
    p = params(num_ants=3 * n, beta=2.0, rho=0.2, cand_k=0, seed=300 + n, nn_order=order,
               heuristic=_abi.ACO_HEURISTIC_DEVICE, fallback=_abi.ACO_FALLBACK_REFERENCE,
               tau0_mode=_abi.ACO_TAU0_DORIGO)
    run_pair(p, d, 6, ctx=f"full row n{n} order{order}")


@pytest.mark.parametrize("k", [0, 16])
def test_subnormal_choice_values_match_oracle(k):
    """beta = 5 on a 100000-wide box with tau0 = 1e-18: choice values down to
    about 1e-44, below the smallest normal float (1.2e-38).  Nothing may flush
    them to zero: the GPU follows the oracle's exact float arithmetic."""
    x, y, d = instance(60, 91, box=100000)
    p = params(num_ants=40, beta=5.0, rho=0.5, cand_k=k, seed=91,
               tau0_mode=_abi.ACO_TAU0_VALUE, tau0=1e-18,
               nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
               fallback=_abi.ACO_FALLBACK_BEST if k else _abi.ACO_FALLBACK_REFERENCE)
    g, q = pair(p, d)
    ch = q.choice()
    tiny = ch[(ch > 0) & (ch < np.float32(1.17549435e-38))]
    assert tiny.size > 0  # the case really holds subnormal choice values
    assert np.array_equal(bits(g.choice_info()), bits(ch))
    for it in range(4):
        g.constructSolution()
        q.iterate()
        assert_same_state(g, q, ctx=f"subnormal k{k} iteration {it}")
    g.close()
    q.close()


def test_cluster_kernel_many_ants_matches_oracle():
    """The cluster kernel with several ant warps per CTA and more ants than
    one pass of the grid holds (n=2100: clusters of 3)."""
    _, _, d = instance(2100, 91, kind="clustered")
    p = params(num_ants=700, beta=2.0, rho=0.1, cand_k=24, seed=91,
               construct_mode=_abi.ACO_CONSTRUCT_CLUSTER, **FAST_MODE)
    run_pair(p, d, 2, ctx="cluster m700")


@pytest.mark.parametrize("apb", [1, 2, 8, 16])
def test_ants_per_block_does_not_change_results(apb):
    _, _, d = instance(66, 4)
    p = params(num_ants=45, beta=2.0, rho=0.2, cand_k=20, seed=4, ants_per_block=apb, **FAST_MODE)
    run_pair(p, d, 3, ctx=f"apb{apb}")


def test_full_size_rank_based_aging_config_matches_oracle():
    """The bench workload (n=1000 clustered, m=1000, RBAS w=6, aging, k=30,
    rho=0.1) for a few iterations: bit-exact with the oracle."""
    _, _, d = instance(1000, 2026, kind="clustered")
    p = params(num_ants=1000, variant=_abi.ACO_RANK_BASED, rank_w=6, aging=1, cand_k=30,
               rho=0.1, beta=2.0, seed=77, **FAST_MODE)
    g, q = pair(p, d, threads=16)
    for it in range(3):
        g.constructSolution()
        q.iterate()
        assert_same_state(g, q, aging=True, ctx=f"full-size iteration {it}")
    tours = g.tours()
    assert is_permutation_rows(tours, 1000)
    assert np.array_equal(tour_lengths(d, tours), g.tour_lengths())


def test_atomic_deposit_within_tolerance_of_fp64():
    """Atomic mode: tours of the first iteration are exact (same tau0); the
    updated pheromone is within 1e-5 relative of the FP64 restatement."""
    _, _, d = instance(300, 8)
    p = params(num_ants=200, beta=2.0, rho=0.1, cand_k=25, seed=8,
               deposit=_abi.ACO_DEPOSIT_ATOMIC, **FAST_MODE)
    g, q = pair(p, d)
    tau0 = g.pheromone().astype(np.float64)
    g.constructSolution()
    q.iterate()
    assert np.array_equal(g.tours(), q.tours())
    lens = g.tour_lengths()
    ref64 = oracle.pheromone_update_f64(tau0, 0.1, g.tours(), lens, np.ones(200))
    tau = g.pheromone().astype(np.float64)
    assert np.max(np.abs(tau - ref64) / ref64) < 1e-5
    # the two mirrored atomics of an edge round in different orders
    assert np.allclose(tau, tau.T, rtol=1e-6, atol=0)


def test_deterministic_deposit_within_tolerance_of_fp64():
    _, _, d = instance(200, 12)
    p = params(num_ants=150, beta=2.0, rho=0.3, cand_k=20, seed=12, **FAST_MODE)
    g = aco.Colony(d, params=p, num_ants=150)
    g.initialize()
    tau = g.pheromone().astype(np.float64)
    for _ in range(5):
        g.constructSolution()
        tau = oracle.pheromone_update_f64(tau, 0.3, g.tours(), g.tour_lengths(), np.ones(150))
        t32 = g.pheromone().astype(np.float64)
        assert np.max(np.abs(t32 - tau) / tau) < 1e-5


def test_large_instance_properties():
    """n=4096 (uniform in [0,100000)^2), m=512, k=32, atomic deposit: tours
    are permutations, lengths match the distances, the best-so-far only
    improves, pheromone stays symmetric within rounding."""
    x, y, d = instance(4096, 31, box=100000)
    p = params(num_ants=512, beta=2.0, rho=0.1, cand_k=32, seed=31,
               deposit=_abi.ACO_DEPOSIT_ATOMIC, **FAST_MODE)
    g = aco.Colony(coords=(x, y), params=p, num_ants=512)
    assert np.array_equal(g.distances(), d)
    g.initialize()
    best = []
    for _ in range(3):
        g.constructSolution()
        best.append(g.getGlobBestDist())
    tours = g.tours()
    assert is_permutation_rows(tours, 4096)
    assert np.array_equal(tour_lengths(d, tours), g.tour_lengths())
    assert best == sorted(best, reverse=True)
    tau = g.pheromone()
    assert np.allclose(tau, tau.T, rtol=1e-6, atol=0)


def test_distances_and_nn_lists_at_scale():
    x, y, d = instance(2000, 5, kind="clustered")
    for order in (_abi.ACO_NN_STABLE, _abi.ACO_NN_REFERENCE_QSORT):
        p = params(num_ants=8, nn_order=order, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                   fallback=_abi.ACO_FALLBACK_BEST, cand_k=0 if order else 48)
        g = aco.Colony(coords=(x, y), params=p, num_ants=8)
        assert np.array_equal(g.distances(), d)
        g.initialize()
        full = oracle.nn_rows(d, order)
        assert np.array_equal(g.nn_list(), full[:, :g.k])
        g.close()


def test_reference_surface():
    _, _, d = instance(30, 1)
    a = aco.AntSystem(d, 30, 12, 1.0, 2.0, 0.5)
    a.initialize()
    t = []
    a.constructSolution(t)
    assert len(t) == 6 and t[1] > 0
    assert a.antSystemName() == "Ant System"
    assert a.getNumAnts() == 12 and a.getNumCities() == 30
    assert a.getNumValidAnts() == 12 and a.getReps() == 0
    tour = a.getTour()
    assert tour.endswith(",") and sorted(int(v) for v in tour[:-1].split(",")) == list(range(1, 31))
    assert abs(a.getRho() - 0.5) < 1e-7 and abs(a.getBeta() - 2.0) < 1e-7
    r = aco.RankBasedAntSystem(d, 30, 12)
    r.setW(40)
    r.initialize()
    assert r.getW() == 30  # w = min(w, n), src/RankBasedAntSystem.cu:31-36
    assert r.antSystemName() == "Rank-based Ant System"
    ag = aco.AntSystem(d, 30, 12, 1.0, 2.0, 0.5, 30, 50, 10, 10, 40, 100)
    ag.initialize()
    ag.constructSolution()
    assert ag.getNumValidAnts() == 12


def test_errors_are_reported_not_fatal():
    _, _, d = instance(20, 1)
    g = aco.Colony(d, params=params(num_ants=5), num_ants=5)
    with pytest.raises(aco.AcoError) as e:
        g.constructSolution()
    assert e.value.status == _abi.ACO_ERR_NOT_INITIALIZED
    with pytest.raises(aco.AcoError):
        aco.Colony(d, params=params(num_ants=0), num_ants=0)
    g.initialize()
    g.constructSolution()
    g.synchronize()
