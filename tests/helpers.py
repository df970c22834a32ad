"""Shared helpers of the test suite: seeded instances and the state
comparisons used by the parity tests."""
import numpy as np

from acogpu_gb300 import _abi, instances


def instance(n, seed, kind="uniform", box=10000):
    if kind == "clustered":
        x, y = instances.clustered_instance(n, box=box, seed=seed)
    else:
        x, y = instances.uniform_instance(n, box=box, seed=seed)
    return x, y, instances.euc2d_distances(x, y)


def params(**kw):
    return _abi.default_params(**kw)


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_same_state(gpu, ora, aging=False, prev_mean=None, ctx=""):
    """Bit-exact comparison of one iteration's observable state."""
    tg, to = gpu.tours(), ora.tours()
    if aging:
        valid = ora.aging()["valid"].astype(bool) if hasattr(ora, "aging") else None
    assert np.array_equal(tg, to), f"{ctx}: tours differ at {np.argwhere(tg != to)[:4].tolist()}"
    assert np.array_equal(gpu.tour_lengths(), ora.lengths()), f"{ctx}: lengths differ"
    assert gpu.getIterBestDist() == ora.iter_best(), f"{ctx}: iteration best differs"
    assert gpu.getGlobBestDist() == ora.glob_best(), f"{ctx}: best-so-far differs"
    tau_g, tau_o = gpu.pheromone(), ora.pheromone()
    bad = np.argwhere(bits(tau_g) != bits(tau_o))
    assert bad.size == 0, f"{ctx}: pheromone differs at {bad[:4].tolist()}"
    assert np.array_equal(gpu.best_tour(), ora.best_tour()), f"{ctx}: best tour differs"
    if aging:
        a, b = gpu.aging_state(), ora.aging()
        for key in ("age", "perf", "valid"):
            assert np.array_equal(a[key], b[key]), f"{ctx}: aging {key} differs"
        assert np.array_equal(bits(a["mean"]), bits(b["mean"])), f"{ctx}: pheromone means differ"
        assert a["isconverged"] == b["isconverged"], f"{ctx}: isconverged differs"
        assert a["globalperformance"] == b["globalperformance"], f"{ctx}: globalperformance"
        assert gpu.getNumValidAnts() == ora.num_valid(), f"{ctx}: valid ants differ"


def is_permutation_rows(tours, n):
    s = np.sort(tours, axis=1)
    return np.array_equal(s, np.broadcast_to(np.arange(n, dtype=s.dtype), s.shape))


def tour_lengths(dist, tours):
    nxt = np.roll(tours, -1, axis=1)
    return dist[tours, nxt].astype(np.int64).sum(axis=1)
