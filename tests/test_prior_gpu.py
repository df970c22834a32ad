"""GPU tests of the learned heuristic prior: features, the MLP's forward and
backward kernels against the CPU oracle, parity of a colony that uses the
prior, and what training buys over the plain method."""
import time

import numpy as np
import pytest
import torch

import oracle
import acogpu_gb300 as aco
from acogpu_gb300 import _abi, instances
from acogpu_gb300.prior import EdgePrior, candidate_heuristic, edge_features
from helpers import assert_same_state
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def colony(n, seed, k=16, m=20, kind="uniform", **kw):
    gen = instances.uniform_instance if kind == "uniform" else instances.clustered_instance
    x, y = gen(n, seed=seed)
    p = _abi.default_params(num_ants=m, cand_k=k, beta=2.0, rho=0.2, seed=seed,
                            nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO, **kw)
    c = aco.Colony(coords=(x, y), params=p, num_ants=m)
    c.initialize()
    return c, x, y, p


def numpy_features(x, y, d, nn):
    n, K = nn.shape
    x = x.astype(np.float32)
    y = y.astype(np.float32)
    d = d.astype(np.float32)
    dk = np.maximum(1.0, d[np.arange(n), nn[:, K - 1]]).astype(np.float32)
    d1 = d[np.arange(n), nn[:, 0]].astype(np.float32)
    mean_dk = np.float32(max(1.0, d[np.arange(n), nn[:, K - 1]].astype(np.float64).mean()))
    out = np.zeros((n * K, 12), np.float32)
    for i in range(n):
        for r in range(K):
            j = nn[i, r]
            row = np.where(nn[j] == i)[0]
            rank = row[0] if len(row) else K
            dij = d[i, j]
            out[i * K + r] = [dij / dk[i], dij / dk[j], r / K, rank / K, (x[j] - x[i]) / dk[i],
                              (y[j] - y[i]) / dk[i], d1[i] / dk[i], d1[j] / dk[j],
                              dij / (d1[i] + d1[j] + 1.0), dk[i] / mean_dk, dk[j] / mean_dk,
                              1.0 if (r < 5 and len(row) and rank < 5) else 0.0]
    return out


def test_edge_features_match_numpy():
    c, x, y, _ = colony(90, 5)
    f = edge_features(c)
    ref = mo.bf16(numpy_features(x, y, c.distances(), c.nn_list()))
    assert np.allclose(f, ref, rtol=1e-2, atol=1e-3)


ENGINES = pytest.mark.parametrize(
    "engine", [_abi.ACO_GEMM_FUSED, _abi.ACO_GEMM_TCGEN05, _abi.ACO_GEMM_MMA_SYNC],
    ids=["fused", "tcgen05", "mma_sync"])


@ENGINES
def test_gradients_match_cpu_oracle(engine):
    """Loss and every parameter gradient of the GPU forward/backward kernels
    against the FP64 oracle (same BF16 rounding points)."""
    c, _, _, _ = colony(80, 9)
    X = edge_features(c)
    rng = np.random.default_rng(1)
    y = (rng.random(len(X)) < 0.2).astype(np.float32)
    pr = EdgePrior(seed=7, engine=engine)
    w = pr.weights()
    lref, gref = mo.loss_and_grads(w, X, y, pos_weight=3.0)
    rp = mo.unpack(gref)
    # repeated: a race in the gradient reduction shows up as a run-to-run change
    for rep in range(4):
        loss, g = pr.loss_and_grads(X, y, pos_weight=3.0)
        assert abs(loss - lref) <= 2e-3 * abs(lref)
        gp = mo.unpack(g)
        for name in ("W1", "b1", "W2", "b2", "w3", "b3"):
            err = np.linalg.norm(gp[name] - rp[name]) / max(1e-12, np.linalg.norm(rp[name]))
            assert err < 1e-2, (rep, name, err)


@pytest.mark.parametrize("E", [1237, 40_000])
def test_fused_pass_over_many_tiles_matches_oracle(E):
    """The fused kernel on a ragged set (the last tile part-filled) and on
    more tiles than SMs (several tiles per CTA, the weight gradients
    accumulated in tensor memory across them); repeated runs are bit-identical
    (partials reduced in a fixed order, no atomics)."""
    rng = np.random.default_rng(E)
    X = mo.bf16(rng.uniform(-1.0, 2.0, size=(E, 12))).astype(np.float32)
    y = (rng.random(E) < 0.15).astype(np.float32)
    pr = EdgePrior(seed=13, engine=_abi.ACO_GEMM_FUSED)
    lref, gref = mo.loss_and_grads(pr.weights(), X, y, pos_weight=4.0)
    rp = mo.unpack(gref)
    first = None
    for rep in range(3):
        loss, g = pr.loss_and_grads(X, y, pos_weight=4.0)
        assert abs(loss - lref) <= 2e-3 * abs(lref)
        gp = mo.unpack(g)
        for name in ("W1", "b1", "W2", "b2", "w3", "b3"):
            err = np.linalg.norm(gp[name] - rp[name]) / max(1e-12, np.linalg.norm(rp[name]))
            assert err < 1e-2, (rep, name, err)
        if first is None:
            first = (loss, g.copy())
        else:
            assert loss == first[0] and np.array_equal(g, first[1])
    p = pr.predict(X)
    assert np.max(np.abs(p - mo.predict(pr.weights(), X))) < 5e-3
    pr.close()


def test_training_engines_agree_and_fused_is_deterministic():
    """Two epochs on the same examples: the fused engine and the two layered
    engines follow the same loss curve (different summation orders only),
    and two fused runs end with bit-identical weights."""
    c, _, _, _ = colony(400, 31, k=20, m=60)
    c.run(20)
    runs = {}
    for name, eng in (("fused", _abi.ACO_GEMM_FUSED), ("fused2", _abi.ACO_GEMM_FUSED),
                      ("tcgen05", _abi.ACO_GEMM_TCGEN05), ("mma_sync", _abi.ACO_GEMM_MMA_SYNC)):
        pr = EdgePrior(seed=21, engine=eng)
        pr.add_examples(c)
        l1 = pr.train(epochs=1, batch=1024, lr=2e-3, seed=4)
        l2 = pr.train(epochs=1, batch=1024, lr=2e-3, seed=5)
        runs[name] = (l1, l2, pr.weights())
        pr.close()
    c.close()
    assert runs["fused"][0] == runs["fused2"][0] and runs["fused"][1] == runs["fused2"][1]
    assert np.array_equal(runs["fused"][2], runs["fused2"][2])
    for name in ("tcgen05", "mma_sync"):
        for k in (0, 1):
            assert abs(runs[name][k] - runs["fused"][k]) <= 0.02 * runs["fused"][k], (name, k)
        dw = np.linalg.norm(runs[name][2] - runs["fused"][2]) / np.linalg.norm(runs["fused"][2])
        assert dw < 2e-2, (name, dw)


@ENGINES
def test_predict_matches_cpu_oracle(engine):
    c, _, _, _ = colony(70, 4)
    X = edge_features(c)
    pr = EdgePrior(seed=3, engine=engine)
    p = pr.predict(X)
    ref = mo.predict(pr.weights(), X)
    assert np.max(np.abs(p - ref)) < 5e-3


def test_colony_with_prior_matches_oracle():
    """With the prior installed the construction stays bit-exact with the
    oracle fed the same candidate heuristic."""
    c, x, y, p = colony(110, 21, k=20, m=40, kind="clustered")
    pr = EdgePrior(seed=11)
    pr.apply(c, floor=0.05)
    eta_nk = candidate_heuristic(c)
    q = oracle.Port(p, c.distances(), threads=4)
    q.initialize()
    q.set_candidate_heuristic(eta_nk)
    for it in range(6):
        c.constructSolution()
        q.iterate()
        assert_same_state(c, q, ctx=f"prior iteration {it}")


def _colony_for(x, y, seed):
    p = _abi.default_params(num_ants=min(len(x), 100), cand_k=20, beta=2.0, rho=0.2, seed=seed,
                            nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO)
    c = aco.Colony(coords=(x, y), params=p, num_ants=p.num_ants)
    c.initialize()
    return c


def _device_seconds(fn):
    torch.cuda.synchronize()
    t = time.perf_counter()
    fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t


def _equal_time_runs(insts, iters, prior, floor=0.05, seed=0):
    """Plain: one untimed iteration, then `iters` timed ones (T_plain).
    Learned: the same untimed iteration, then the prior's inference
    (features, MLP, heuristic update; T_infer) charged to the same budget,
    which buys floor((T_plain - T_infer) / t_iter) iterations, t_iter =
    T_plain / iters from the plain run of the same instance."""
    plain, learned, spent = [], [], []
    for i, (x, y) in enumerate(insts):
        c = _colony_for(x, y, seed + i)
        c.run(1)  # warm-up, not counted
        t_plain = _device_seconds(lambda: c.run(iters))
        plain.append(c.getGlobBestDist())
        c.close()
        c = _colony_for(x, y, seed + i)
        c.run(1)
        t_infer = _device_seconds(lambda: prior.apply(c, floor))
        budget = min(iters, max(0, int((t_plain - t_infer) / (t_plain / iters))))
        c.run(budget)
        learned.append(c.getGlobBestDist())
        spent.append((t_infer, budget))
        c.close()
    return np.array(plain, np.float64), np.array(learned, np.float64), spent


def test_training_learns_and_the_prior_helps():
    """Train on labels from the plain method's best tours, then compare the
    plain method with and without the prior at equal GPU time on fresh
    instances (the learned arm pays for its inference in iterations)."""
    train = [instances.uniform_instance(int(n), seed=500 + i) if i % 2 == 0 else
             instances.clustered_instance(int(n), seed=500 + i)
             for i, n in enumerate(np.linspace(100, 200, 24).astype(int))]
    p = _abi.default_params(cand_k=20, beta=2.0, rho=0.2, seed=99, nn_order=_abi.ACO_NN_STABLE,
                            heuristic=_abi.ACO_HEURISTIC_DEVICE, fallback=_abi.ACO_FALLBACK_BEST,
                            tau0_mode=_abi.ACO_TAU0_DORIGO)
    b = aco.Batch(train, params=p, num_ants=100)
    b.initialize()
    b.run(60)
    b.synchronize()
    pr = EdgePrior(seed=5)
    for i in range(len(train)):
        pr.add_examples(b.colony(i))
    E, pos = pr.num_examples()
    assert E == sum(len(x) for x, _ in train) * 20 and 0 < pos < E
    first = pr.train(epochs=1, batch=4096, lr=2e-3, seed=1)
    last = pr.train(epochs=8, batch=4096, lr=2e-3, seed=2)
    assert last < first
    b.close()
    test = [instances.uniform_instance(300, seed=900 + i) for i in range(6)]
    plain, learned, spent = _equal_time_runs(test, 30, pr, seed=3)
    assert all(b >= 1 for _, b in spent), spent
    assert learned.mean() < plain.mean(), (learned.mean(), plain.mean(), spent)
