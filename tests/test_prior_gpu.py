"""GPU tests of the learned heuristic prior: features, the MLP's forward and
backward kernels against the CPU oracle, parity of a colony that uses the
prior, and what training buys over the plain method."""
import numpy as np
import pytest

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


ENGINES = pytest.mark.parametrize("engine", [_abi.ACO_GEMM_TCGEN05, _abi.ACO_GEMM_MMA_SYNC],
                                  ids=["tcgen05", "mma_sync"])


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


def _plain_runs(insts, iters, prior=None, floor=0.05, seed=0):
    best = []
    for i, (x, y) in enumerate(insts):
        p = _abi.default_params(num_ants=min(len(x), 100), cand_k=20, beta=2.0, rho=0.2,
                                seed=seed + i, nn_order=_abi.ACO_NN_STABLE,
                                heuristic=_abi.ACO_HEURISTIC_DEVICE,
                                fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO)
        c = aco.Colony(coords=(x, y), params=p, num_ants=p.num_ants)
        c.initialize()
        if prior is not None:
            prior.apply(c, floor)
        c.run(iters)
        best.append(c.getGlobBestDist())
        c.close()
    return np.array(best, dtype=np.float64)


def test_training_learns_and_the_prior_helps():
    """Train on labels from the plain method's best tours, then compare the
    plain method with and without the prior at the same iteration budget on
    fresh instances."""
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
    plain = _plain_runs(test, 10, seed=3)
    learned = _plain_runs(test, 10, prior=pr, seed=3)
    assert learned.mean() < plain.mean(), (learned.mean(), plain.mean())
