"""GPU parity over whole configured runs (not a few iterations):

* C1 as specified -- plain AS, n = 100, m = 100, beta 2, rho 0.5, full-row
  roulette, 1000 iterations -- against the running digest recorded from the
  compiled reference (tests/golden/c1_as_n100_1000iters.json);
* C2 at full size -- rank-based AS with aging, n = 1000 clustered, m = 1000,
  w = 6, k = 30, rho 0.1 -- for all 500 iterations against the port, which
  covers convergence, the blending recruits and retire/recruit at the bench
  size;
* the parity-mode batch of the bench (the reference's own algorithm with
  aging on n = 1000 instances) and a stratified sample of the uneven batch
  (C4: n from 50 to 2000, k = 20), every instance against its own port;
* a checkpoint resumed into a fresh colony, and the broker variant, both
  against the port.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
import acogpu_gb300 as aco
from acogpu_gb300 import _abi, instances
from helpers import assert_same_state, bits, instance

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_STEP = np.uint64(0x9E3779B97F4A7C15)
THREADS = os.cpu_count() or 4


def chain_digest(h, tours, lengths, tau):
    m = hashlib.sha256(h)
    m.update(np.ascontiguousarray(tours, dtype=np.int32).tobytes())
    m.update(np.ascontiguousarray(lengths, dtype=np.int64).tobytes())
    m.update(np.ascontiguousarray(tau, dtype=np.float32).tobytes())
    return m.digest()


def instance_params(p, i):
    q = _abi.AcoParams.from_buffer_copy(p)
    with np.errstate(over="ignore"):
        q.seed = int(np.uint64(p.seed) + np.uint64(i) * GOLDEN_STEP)
    return q


def test_c1_whole_run_matches_the_reference_digest():
    """1000 iterations on the GPU (the long-row kernel, k = n = 100): every
    iteration's best and the running digest of tours, lengths and pheromone
    at the checkpoints equal the compiled reference's run."""
    c = json.load(open(os.path.join(GOLDEN, "c1_as_n100_1000iters.json")))
    x, y = instances.uniform_instance(c["n"], seed=c["seed"])
    d = instances.euc2d_distances(x, y)
    p = _abi.default_params(num_ants=c["m"], beta=c["beta"], rho=c["rho"], aging=0,
                            seed=1000 + c["seed"], nn_order=_abi.ACO_NN_REFERENCE_QSORT)
    g = aco.Colony(d, params=p, num_ants=c["m"])
    g.initialize()
    h = b""
    for it in range(1, c["iters"] + 1):
        g.constructSolution()
        h = chain_digest(h, g.tours(), g.tour_lengths(), g.pheromone())
        assert g.getIterBestDist() == c["iter_best"][it - 1], f"iteration {it}: iteration best"
        assert g.getGlobBestDist() == c["glob_best"][it - 1], f"iteration {it}: best so far"
        if str(it) in c["digests"]:
            assert h.hex() == c["digests"][str(it)], f"iteration {it}: digest"
    assert [int(v) for v in g.best_tour()] == c["best_tour"]
    g.close()


def test_c2_all_500_iterations_match_the_port():
    """C2 at full size for its whole run: the integer lengths of every ant in
    every iteration, and the full state (tours, pheromone bits, bests, aging
    counters) every 50 iterations and at the end."""
    x, y = instances.clustered_instance(1000, seed=2026)
    d = instances.euc2d_distances(x, y)
    p = _abi.default_params(num_ants=1000, variant=_abi.ACO_RANK_BASED, rank_w=6, aging=1,
                            cand_k=30, rho=0.1, beta=2.0, nn_order=_abi.ACO_NN_STABLE,
                            heuristic=_abi.ACO_HEURISTIC_DEVICE,
                            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO,
                            deposit=_abi.ACO_DEPOSIT_DETERMINISTIC, seed=1234)
    g = aco.Colony(d, params=p, num_ants=1000)
    g.initialize()
    q = oracle.Port(p, d, threads=THREADS)
    q.initialize()
    converged_at = None
    for it in range(1, 501):
        g.constructSolution()
        q.iterate()
        assert np.array_equal(g.tour_lengths(), q.lengths()), f"iteration {it}: lengths"
        if converged_at is None and q.aging()["isconverged"]:
            converged_at = it
        if it % 50 == 0 or it == 500:
            assert_same_state(g, q, aging=True, ctx=f"iteration {it}")
    assert converged_at is not None and converged_at < 500  # blending ants were exercised
    g.close()
    q.close()


def _batch_vs_ports(insts, p, cap, iters, ctx):
    b = aco.Batch(insts, params=p, num_ants=cap)
    b.initialize()
    ports = []
    for i, (x, y) in enumerate(insts):
        qi = instance_params(p, i)
        qi.num_ants = min(cap, len(x))
        q = oracle.Port(qi, instances.euc2d_distances(x, y), threads=THREADS)
        q.initialize()
        ports.append(q)
    for it in range(iters):
        b.run(1)
        b.synchronize()
        for i, q in enumerate(ports):
            q.iterate()
            assert_same_state(b.colony(i), q, aging=bool(p.aging),
                              ctx=f"{ctx}: instance {i} (n={len(insts[i][0])}) iteration {it}")
    for q in ports:
        q.close()
    b.close()


def test_parity_batch_matches_the_port():
    """The bench's parity-mode batch (full rows in the reference nn order,
    libm heuristic, reference fallback, tau0 1e-6, aging), three instances
    of n = 1000, four iterations, every instance's whole state."""
    insts = [instances.clustered_instance(1000, seed=2026 + i) for i in range(3)]
    p = _abi.default_params(num_ants=1000, aging=1, cand_k=0, rho=0.1, beta=2.0, seed=1234)
    _batch_vs_ports(insts, p, 1000, 4, "parity batch")


def test_uneven_batch_sample_matches_the_port():
    """A stratified sample of the uneven batch (C4): sizes from 50 to 2000,
    uniform and clustered alternating, k = 20, AS; three iterations, every
    instance against its own port."""
    sizes = [50, 64, 90, 128, 181, 256, 362, 512, 600, 724, 900, 1024, 1300, 1448, 1700, 2000]
    insts = [(instances.uniform_instance if i % 2 == 0 else instances.clustered_instance)(
        n, seed=10_000 + i) for i, n in enumerate(sizes)]
    p = _abi.default_params(cand_k=20, rho=0.1, beta=2.0, nn_order=_abi.ACO_NN_STABLE,
                            heuristic=_abi.ACO_HEURISTIC_DEVICE, fallback=_abi.ACO_FALLBACK_BEST,
                            tau0_mode=_abi.ACO_TAU0_DORIGO, seed=4321)
    _batch_vs_ports(insts, p, 1024, 3, "uneven batch")


@pytest.mark.parametrize("variant,aging,cand_k", [(_abi.ACO_RANK_BASED, 1, 30),
                                                  (_abi.ACO_ANT_SYSTEM, 1, 0)])
def test_checkpoint_resume_continues_like_the_port(tmp_path, variant, aging, cand_k):
    """A colony saved after 6 iterations and loaded into a fresh colony goes
    on exactly like the port that simply kept running."""
    _, _, d = instance(300, 61, kind="clustered")
    p = _abi.default_params(num_ants=120, variant=variant, rank_w=6, aging=aging, cand_k=cand_k,
                            rho=0.2, beta=2.0, seed=61,
                            fallback=(_abi.ACO_FALLBACK_BEST if cand_k else
                                      _abi.ACO_FALLBACK_REFERENCE))
    (p.min_retirement_age, p.max_retirement_age, p.global_performance,
     p.min_population_limit) = (3, 6, 2, 40)
    a = aco.Colony(d, params=p, num_ants=p.num_ants)
    a.initialize()
    q = oracle.Port(p, d, threads=THREADS)
    q.initialize()
    for _ in range(6):
        a.constructSolution()
        q.iterate()
    path = tmp_path / "colony.ckpt"
    a.save(path)
    a.close()
    b = aco.Colony(d, params=p, num_ants=p.num_ants)
    b.initialize()
    b.load(path)
    for it in range(8):
        b.constructSolution()
        q.iterate()
        assert_same_state(b, q, aging=bool(aging), ctx=f"iteration {it} after resume")
    b.close()
    q.close()


def test_broker_variant_changes_nothing():
    """The broker/nobroker variant is a flag with no behaviour in the
    reference (inc/broker/parallel.h:3, inc/Colony.h:142-149): broker = 1
    and broker = 0 colonies and the port agree bit for bit."""
    _, _, d = instance(150, 62)
    base = dict(num_ants=60, aging=1, cand_k=0, rho=0.3, beta=2.0, seed=62)
    g0 = aco.Colony(d, params=_abi.default_params(broker=0, **base), num_ants=60)
    g1 = aco.Colony(d, params=_abi.default_params(broker=1, **base), num_ants=60)
    g0.initialize()
    g1.initialize()
    q = oracle.Port(_abi.default_params(broker=1, **base), d, threads=THREADS)
    q.initialize()
    for it in range(12):
        g0.constructSolution()
        g1.constructSolution()
        q.iterate()
        assert_same_state(g1, q, aging=True, ctx=f"broker=1 iteration {it}")
        assert np.array_equal(g0.tours(), g1.tours())
        assert np.array_equal(bits(g0.pheromone()), bits(g1.pheromone()))
    for g in (g0, g1):
        g.close()
    q.close()
