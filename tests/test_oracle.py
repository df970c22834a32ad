"""CPU tests of the oracle: pinned against the reference's own CPU path
(golden fixtures, and the reference compiled in place when its sources are
present), plus the random stream and the instance generators."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from acogpu_gb300 import _abi, instances
from helpers import bits, instance, params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = json.load(open(os.path.join(GOLDEN, "cases.json")))


def golden_params(meta):
    p = params(num_ants=meta["m"], beta=meta["beta"], rho=meta["rho"], aging=meta["aging"],
               seed=meta["seed_stream"],
               nn_order=_abi.ACO_NN_STABLE if meta["stable"] else _abi.ACO_NN_REFERENCE_QSORT)
    if meta["aging"]:
        (p.min_retirement_age, p.max_retirement_age, p.local_performance, p.global_performance,
         p.min_population_limit, p.max_population_limit) = meta["six"]
    return p


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_matches_golden(name):
    """The C restatement reproduces the reference's recorded run exactly."""
    meta = CASES[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = oracle.distances(g["x"], g["y"])
    assert np.array_equal(d, g["dist"])
    q = oracle.Port(golden_params(meta), d, threads=2)
    q.initialize()
    assert np.array_equal(q.nn(), g["nn"])
    assert np.array_equal(bits(q.heuristic()), bits(g["eta"]))
    for it in range(meta["iters"]):
        q.iterate()
        assert np.array_equal(q.tours(), g["tours"][it]), f"iteration {it}: tours"
        assert np.array_equal(q.lengths(), g["lengths"][it]), f"iteration {it}: lengths"
        assert q.iter_best() == g["iter_best"][it]
        assert q.glob_best() == g["glob_best"][it]
        assert q.num_valid() == g["num_valid"][it]
        h = hashlib.sha256(q.pheromone().tobytes()).hexdigest()
        assert h == meta["tau_hashes"][it], f"iteration {it}: pheromone"
    assert np.array_equal(q.best_tour(), g["best_tour"])


def c1_digest_case():
    """The whole-run digest recorded from the compiled reference (C1: plain
    AS, n = 100, m = 100, beta 2, rho 0.5, full rows, 1000 iterations)."""
    return json.load(open(os.path.join(GOLDEN, "c1_as_n100_1000iters.json")))


def c1_digest_params(c):
    return _abi.default_params(num_ants=c["m"], beta=c["beta"], rho=c["rho"], aging=0,
                               seed=1000 + c["seed"], nn_order=_abi.ACO_NN_REFERENCE_QSORT)


def chain_digest(h, tours, lengths, tau):
    m = hashlib.sha256(h)
    m.update(np.ascontiguousarray(tours, dtype=np.int32).tobytes())
    m.update(np.ascontiguousarray(lengths, dtype=np.int64).tobytes())
    m.update(np.ascontiguousarray(tau, dtype=np.float32).tobytes())
    return m.digest()


def test_port_reproduces_the_whole_c1_run():
    """All 1000 iterations of C1 on the port: every iteration's best, and the
    running digest of tours, lengths and pheromone at the checkpoints, equal
    the compiled reference's."""
    c = c1_digest_case()
    x, y = instances.uniform_instance(c["n"], seed=c["seed"])
    q = oracle.Port(c1_digest_params(c), oracle.distances(x, y), threads=4)
    q.initialize()
    h = b""
    for it in range(1, c["iters"] + 1):
        q.iterate()
        h = chain_digest(h, q.tours(), q.lengths(), q.pheromone())
        assert q.iter_best() == c["iter_best"][it - 1], f"iteration {it}: iteration best"
        assert q.glob_best() == c["glob_best"][it - 1], f"iteration {it}: best so far"
        if str(it) in c["digests"]:
            assert h.hex() == c["digests"][str(it)], f"iteration {it}: digest"
    assert [int(v) for v in q.best_tour()] == c["best_tour"]
    q.close()


needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference sources absent")


@needs_ref
@pytest.mark.parametrize("n,m,aging,stable,beta,rho,iters,seed", [
    (30, 12, 0, False, 5.0, 0.1, 6, 21),
    (70, 40, 0, True, 2.0, 0.5, 6, 22),
    (45, 30, 1, False, 2.0, 0.2, 30, 23),
])
def test_port_matches_compiled_reference(n, m, aging, stable, beta, rho, iters, seed):
    x, y, d = instance(n, seed, kind="clustered" if seed % 2 else "uniform")
    p = params(num_ants=m, beta=beta, rho=rho, aging=aging, seed=seed,
               nn_order=_abi.ACO_NN_STABLE if stable else _abi.ACO_NN_REFERENCE_QSORT)
    if aging:
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (3, 6, 2, m // 2)
    ref = oracle.Ref(p, d, stable_nn=stable)
    ref.initialize()
    q = oracle.Port(p, d, threads=3)
    q.initialize()
    assert np.array_equal(ref.nn(), q.nn())
    assert np.array_equal(bits(ref.heuristic()), bits(q.heuristic()))
    for it in range(iters):
        mean_before = q.aging()["mean"].copy() if aging else None
        ref.iterate()
        q.iterate()
        assert np.array_equal(ref.tours(), q.tours()), it
        assert np.array_equal(ref.lengths(), q.lengths()), it
        assert np.array_equal(bits(ref.pheromone()), bits(q.pheromone())), it
        assert (ref.iter_best(), ref.glob_best()) == (q.iter_best(), q.glob_best())
        if aging:
            a, b = ref.aging_state(), q.aging()
            # the reference computes the row means at the start of an
            # iteration, the port at the end of the previous one
            assert np.array_equal(bits(a["mean"]), bits(mean_before))
            for key in ("age", "perf", "valid"):
                assert np.array_equal(a[key], b[key])
            assert a["isconverged"] == b["isconverged"]
    ref.close()


@needs_ref
@pytest.mark.parametrize("stable,aging", [(False, 0), (True, 0), (False, 1)])
def test_port_matches_compiled_reference_with_coincident_cities(stable, aging):
    """Cities moved onto one point in triples: distance 0, an infinite
    heuristic and choice value, row sums of +inf.  The reference's walk then
    runs past the row into select_local_best (or stops at the first
    candidate for u*S = NaN); the port must follow it exactly -- this pins
    the engine's handling of infinite weights to the reference itself."""
    from acogpu_gb300 import instances
    n, m = 48, 24
    x, y = instances.uniform_instance(n, seed=77)
    x, y = np.array(x), np.array(y)
    pick = np.random.default_rng(77).choice(n, 12, replace=False).reshape(4, 3)
    for a, b, c in pick:
        x[b] = x[c] = x[a]
        y[b] = y[c] = y[a]
    d = instances.euc2d_distances(x, y)
    assert (d[~np.eye(n, dtype=bool)] == 0).sum() >= 24
    p = params(num_ants=m, beta=2.0, rho=0.2, seed=77, aging=aging,
               nn_order=_abi.ACO_NN_STABLE if stable else _abi.ACO_NN_REFERENCE_QSORT)
    if aging:
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (3, 5, 2, m // 2)
    ref = oracle.Ref(p, d, stable_nn=stable)
    ref.initialize()
    q = oracle.Port(p, d, threads=3)
    q.initialize()
    assert np.isinf(q.heuristic()).any()
    for it in range(12 if aging else 8):
        ref.iterate()
        q.iterate()
        assert np.array_equal(ref.tours(), q.tours()), it
        assert np.array_equal(ref.lengths(), q.lengths()), it
        assert np.array_equal(bits(ref.pheromone()), bits(q.pheromone())), it
        assert (ref.iter_best(), ref.glob_best()) == (q.iter_best(), q.glob_best())
        if aging:
            a, b = ref.aging_state(), q.aging()
            for key in ("age", "perf", "valid"):
                assert np.array_equal(a[key], b[key]), (it, key)
    ref.close()
    q.close()


@needs_ref
def test_reference_quicksort_order_differs_from_stable():
    """Ties in rounded distances make the reference's quicksort order differ
    from the stable order; both orders are reproduced."""
    x, y, d = instance(300, 5)
    ref = oracle.Ref(params(num_ants=4), d)
    ref.initialize()
    q = oracle.nn_rows(d, _abi.ACO_NN_REFERENCE_QSORT)
    s = oracle.nn_rows(d, _abi.ACO_NN_STABLE)
    assert np.array_equal(ref.nn(), q)
    assert not np.array_equal(q, s)
    assert np.array_equal(np.sort(q, axis=1), np.sort(s, axis=1))


def test_distances_match_numpy_restatement():
    for seed, box in ((1, 10000), (2, 100000)):
        x, y = instances.uniform_instance(257, box=box, seed=seed)
        assert np.array_equal(oracle.distances(x, y), instances.euc2d_distances(x, y))


def test_stable_nn_rows_are_sorted_by_distance_then_index():
    _, _, d = instance(200, 3)
    nn = oracle.nn_rows(d, _abi.ACO_NN_STABLE)
    for r in range(0, 200, 17):
        keys = d[r, nn[r]].astype(np.int64) * 1000 + nn[r]
        assert np.all(np.diff(keys) > 0)
        assert nn[r, -1] == r  # the diagonal (MAX) sorts last


def test_heuristic_modes():
    """Device mode is the correctly rounded (1/d)^beta; libm mode is the
    reference's powf and differs from it in a few ulp-level cases."""
    from fractions import Fraction
    diffs = 0
    for d in list(range(1, 400)) + [1414, 9999, 14142]:
        x = np.float32(1.0) / np.float32(d)
        exact = Fraction(float(x)) ** 2
        dev = oracle.heuristic(d, 2.0, _abi.ACO_HEURISTIC_DEVICE)
        cands = [np.nextafter(np.float32(float(exact)), np.float32(0)), np.float32(float(exact)),
                 np.nextafter(np.float32(float(exact)), np.float32(1))]
        best = min(cands, key=lambda c: abs(Fraction(float(c)) - exact))
        assert np.float32(dev) == best, d
        lib = oracle.heuristic(d, 2.0, _abi.ACO_HEURISTIC_LIBM)
        diffs += np.float32(lib) != np.float32(dev)
        assert abs(float(lib) - float(dev)) <= abs(float(dev)) * 2.0 ** -23
    assert oracle.heuristic(0x7FFFFFFF, 2.0, _abi.ACO_HEURISTIC_DEVICE) == 0.0
    assert np.isinf(oracle.heuristic(0, 2.0, _abi.ACO_HEURISTIC_DEVICE))


def test_rng_stream_properties():
    """u is a pure function of (seed, iteration, ant, step), in (0, 1), and
    (long)(u * n) < n for every n."""
    from acogpu_gb300 import rng
    u = rng.uniform_grid(1234, 7, np.arange(2000), np.arange(64))
    assert u.shape == (2000, 64)
    assert u.min() > 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01
    assert np.array_equal(u, rng.uniform_grid(1234, 7, np.arange(2000), np.arange(64)))
    assert not np.array_equal(u, rng.uniform_grid(1234, 8, np.arange(2000), np.arange(64)))
    top = np.float32(1.0) - np.float32(2.0 ** -24)
    for n in (3, 7, 100, 1000, 4095, 65537, 2 ** 21 - 1):
        assert int(np.float32(top) * np.float32(n)) < n


def test_instances_are_seeded():
    a = instances.clustered_instance(500, seed=4)
    b = instances.clustered_instance(500, seed=4)
    assert all(np.array_equal(p, q) for p, q in zip(a, b))
    x, y = a
    assert x.min() >= 0 and x.max() < 10000 and np.all(x == np.round(x))
    s = instances.batch_sizes(512)
    assert s.min() >= 50 and s.max() <= 2000


def test_rank_based_update_uses_ranked_ants_and_best_so_far():
    """The port's rank-based update deposits (w-r)/L on the w-1 best ants and
    w/L_gb on the best-so-far tour (checked against an FP64 restatement)."""
    _, _, d = instance(40, 9)
    p = params(num_ants=12, variant=_abi.ACO_RANK_BASED, rank_w=4, beta=2.0, rho=0.25, seed=5,
               nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE)
    q = oracle.Port(p, d)
    q.initialize()
    q.iterate()
    tau0 = np.full((40, 40), np.float64(q.tau0()))
    tours, lens = q.tours(), q.lengths()
    order = sorted(range(12), key=lambda k: (lens[k], k))[:3]
    srcs = [tours[k] for k in order] + [q.best_tour()]
    ls = [lens[k] for k in order] + [q.glob_best()]
    w = [3.0, 2.0, 1.0, 4.0]
    ref64 = oracle.pheromone_update_f64(tau0, 0.25, np.stack(srcs), np.array(ls), np.array(w))
    tau = q.pheromone().astype(np.float64)
    assert np.max(np.abs(tau - ref64) / ref64) < 1e-5


def test_mlp_oracle_backward_matches_finite_differences():
    """The MLP oracle's analytic gradient (exact arithmetic) against central
    differences of its own loss."""
    from oracle import mlp_oracle as mo
    rng = np.random.default_rng(3)
    X = rng.normal(size=(40, 12))
    y = (rng.random(40) < 0.3).astype(np.float64)
    w = np.concatenate([rng.normal(size=128 * 12) * 0.3, rng.normal(size=128) * 0.1,
                        rng.normal(size=128 * 128) * 0.1, rng.normal(size=128) * 0.1,
                        rng.normal(size=128) * 0.2, [0.05]])
    loss, g = mo.loss_and_grads(w, X, y, pos_weight=3.0, exact=True)
    idx = rng.choice(len(w), 60, replace=False)
    for i in idx:
        e = np.zeros_like(w)
        e[i] = 1e-6
        num = (mo.loss_and_grads(w + e, X, y, 3.0, True)[0] -
               mo.loss_and_grads(w - e, X, y, 3.0, True)[0]) / 2e-6
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(num), (i, num, g[i])
