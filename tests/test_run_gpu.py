"""GPU tests of the run loop (aco_execute, the reference's TSP::execute):
its termination rules, the per-iteration statistics and summary, parity of
the best-length sequence with the oracle, and a TSPLIB file driven end to
end."""
import numpy as np
import pytest

import oracle
import acogpu_gb300 as aco
from acogpu_gb300 import _abi, instances, tsplib
from acogpu_gb300.run import TSP
from helpers import instance

pytestmark = pytest.mark.gpu

FAST = dict(nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO)


def colony(n=120, m=40, seed=8, **kw):
    _, _, d = instance(n, seed, kind="clustered")
    p = _abi.default_params(num_ants=m, beta=2.0, rho=0.2, cand_k=20, seed=seed, **FAST, **kw)
    return aco.Colony(d, params=p, num_ants=m), d, p


def test_iteration_limit_statistics_and_summary():
    c, d, p = colony()
    stats, summary = TSP(max_iter=9).execute(c, calcdisttime=1.5)
    assert summary["numiter"] == 9 and len(stats) == 9
    assert [s["iter"] for s in stats] == list(range(9))
    ib = np.array([s["iterbest"] for s in stats])
    gb = np.array([s["globalbest"] for s in stats])
    assert np.array_equal(gb, np.minimum.accumulate(ib))
    assert all(s["ants"] == 40 for s in stats)
    it = np.array([s["t_itertime"] for s in stats], np.float32)
    parts = np.array([[s[k] for k in ("t_inittour", "t_tour", "t_antdist", "t_evapphoremone",
                                      "t_updatephoremone", "t_computeprob")] for s in stats],
                     np.float32)
    assert np.all(it > 0) and np.allclose(it, parts.sum(axis=1), rtol=1e-5)
    assert np.allclose([s["t_globaltime"] for s in stats], np.cumsum(it), rtol=1e-4)
    assert summary["numcities"] == 120 and summary["numants"] == 40
    assert summary["d_calulated"] == np.float32(gb[-1]) and summary["d_optimal"] == -1
    err = (np.float32(gb[-1]) - np.float32(-1)) / np.float32(-1) * np.float32(100)
    assert summary["d_error"] == pytest.approx(float(err), rel=1e-6)
    assert summary["t_distcalc"] == pytest.approx(1.5) and summary["t_inittime"] > 0
    assert summary["p_beta"] == pytest.approx(2.0) and summary["p_rho"] == pytest.approx(0.2)
    assert summary["t_totaltime"] == pytest.approx(float(it.sum()), rel=1e-4)
    c.close()


@pytest.mark.parametrize("limits,expected", [
    (dict(max_iter=50, optimum=10**9), 1),   # the first iteration beats the optimum
    (dict(max_iter=50, max_time=0), 0),      # no time left before the first iteration
    (dict(max_iter=50, max_reps=0), 0),      # reps is 0 >= 0
    (dict(max_iter=0), 0),
])
def test_termination_rules(limits, expected):
    c, _, _ = colony(n=80, m=20)
    stats, summary = TSP(**limits).execute(c)
    assert summary["numiter"] == expected == len(stats)
    c.close()


def test_time_limit_stops_the_loop():
    c, _, _ = colony(n=200, m=200)
    stats, summary = TSP(max_iter=100000, max_time=5).execute(c, max_stats=100000)
    assert 0 < summary["numiter"] < 100000
    assert summary["t_totaltime"] >= 5
    assert stats[-2]["t_globaltime"] < 5  # the loop stopped at the first check past the limit
    c.close()


def test_best_sequence_matches_oracle():
    c, d, p = colony(n=150, m=60, seed=12)
    stats, _ = TSP(max_iter=7).execute(c)
    q = oracle.Port(p, d, threads=8)
    q.initialize()
    for s in stats:
        q.iterate()
        assert s["iterbest"] == q.iter_best() and s["globalbest"] == q.glob_best()
    q.close()
    c.close()


def test_tsplib_file_end_to_end(tmp_path):
    x, y = instances.uniform_instance(400, seed=21)
    body = "".join(f"{i + 1} {int(a)} {int(b)}\n" for i, (a, b) in enumerate(zip(x, y)))
    path = tmp_path / "u400.tsp"
    path.write_text("NAME : u400\nTYPE : TSP\nDIMENSION : 400\nEDGE_WEIGHT_TYPE : EUC_2D\n"
                    f"NODE_COORD_SECTION\n{body}EOF\n")
    p = _abi.default_params(num_ants=64, beta=2.0, rho=0.2, cand_k=20, seed=4, **FAST)
    c = tsplib.colony(path, params=p)
    assert np.array_equal(c.distances(), instances.euc2d_distances(x, y))
    stats, summary = TSP(max_iter=5).execute(c)
    assert summary["numiter"] == 5 and summary["numcities"] == 400
    tour = c.getTour()
    assert sorted(int(t) for t in tour.strip(",").split(",")) == list(range(1, 401))
    c.close()
