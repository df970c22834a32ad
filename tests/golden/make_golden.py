"""Generate the golden fixtures from the reference's own CPU AntSystem.

Run in a checkout that has the reference sources (ACO_REFERENCE_DIR, or a
`reference` directory beside this repository): it builds oracle/_ref with oracle/Makefile, runs the
unmodified reference path with the injected random stream on small seeded
instances and records, per iteration, the tours, lengths and best values and
a hash of the pheromone matrix.  The fixtures pin the oracle and the GPU
path on machines where the reference is absent.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from acogpu_gb300 import _abi, instances  # noqa: E402

CASES = [
    # name, n, m, kind, seed, aging, stable_nn, beta, rho, iterations, aging params
    dict(name="as_noaging_n48", n=48, m=24, kind="uniform", seed=11, aging=0, stable=False,
         beta=2.0, rho=0.5, iters=12),
    dict(name="as_noaging_beta5_n64", n=64, m=32, kind="clustered", seed=12, aging=0,
         stable=False, beta=5.0, rho=0.1, iters=8),
    dict(name="as_noaging_stable_n40", n=40, m=20, kind="uniform", seed=13, aging=0, stable=True,
         beta=2.0, rho=0.5, iters=10),
    dict(name="as_aging_n40", n=40, m=30, kind="uniform", seed=14, aging=1, stable=False,
         beta=2.0, rho=0.3, iters=40, six=(3, 5, 10, 2, 15, 100)),
    dict(name="as_aging_defaults_n56", n=56, m=24, kind="clustered", seed=15, aging=1,
         stable=False, beta=5.0, rho=0.1, iters=60, six=(30, 50, 10, 10, 40, 100)),
]


def tau_hash(tau):
    return hashlib.sha256(np.ascontiguousarray(tau, dtype=np.float32).tobytes()).hexdigest()


def make_case(c):
    if c["kind"] == "clustered":
        x, y = instances.clustered_instance(c["n"], seed=c["seed"])
    else:
        x, y = instances.uniform_instance(c["n"], seed=c["seed"])
    d = oracle.distances(x, y)
    p = _abi.default_params(num_ants=c["m"], beta=c["beta"], rho=c["rho"], aging=c["aging"],
                            seed=1000 + c["seed"],
                            nn_order=_abi.ACO_NN_STABLE if c["stable"] else
                            _abi.ACO_NN_REFERENCE_QSORT)
    if c["aging"]:
        (p.min_retirement_age, p.max_retirement_age, p.local_performance, p.global_performance,
         p.min_population_limit, p.max_population_limit) = c["six"]
    ref = oracle.Ref(p, d, stable_nn=c["stable"])
    ref.initialize()
    out = dict(x=x, y=y, dist=d, nn=ref.nn(), eta=ref.heuristic(), tau0=ref.pheromone())
    tours, lens, ib, gb, th, nv = [], [], [], [], [], []
    for _ in range(c["iters"]):
        ref.iterate()
        tours.append(ref.tours())
        lens.append(ref.lengths())
        ib.append(ref.iter_best())
        gb.append(ref.glob_best())
        th.append(tau_hash(ref.pheromone()))
        nv.append(ref.num_valid())
    out.update(tours=np.stack(tours), lengths=np.stack(lens), iter_best=np.array(ib, np.int64),
               glob_best=np.array(gb, np.int64), num_valid=np.array(nv, np.int32),
               tau_final=ref.pheromone(), best_tour=ref.best_tour())
    if c["aging"]:
        a = ref.aging_state()
        out.update(age=a["age"], valid=a["valid"], isconverged=np.int32(a["isconverged"]))
    meta = {k: v for k, v in c.items()}
    meta["seed_stream"] = int(p.seed)
    meta["tau_hashes"] = th
    ref.close()
    return out, meta


# The first configuration of the benchmark plan, run as specified: plain Ant
# System, n = 100 cities with integer coordinates uniform in [0, 10000)^2,
# m = 100 ants, alpha 1, beta 2, rho 0.5, full-row roulette, 1000
# iterations, no aging.  Recorded as digests, not arrays.
DIGEST = dict(name="c1_as_n100_1000iters", n=100, m=100, seed=100, beta=2.0, rho=0.5,
              iters=1000, checkpoints=[1, 2, 10, 50, 100, 250, 500, 750, 1000])


def chain_digest(h, tours, lengths, tau):
    """Running SHA-256 over the iterations: h_i = H(h_{i-1} | tours | lengths | tau)."""
    m = hashlib.sha256(h)
    m.update(np.ascontiguousarray(tours, dtype=np.int32).tobytes())
    m.update(np.ascontiguousarray(lengths, dtype=np.int64).tobytes())
    m.update(np.ascontiguousarray(tau, dtype=np.float32).tobytes())
    return m.digest()


def digest_params(c):
    return _abi.default_params(num_ants=c["m"], beta=c["beta"], rho=c["rho"], aging=0,
                               seed=1000 + c["seed"], nn_order=_abi.ACO_NN_REFERENCE_QSORT)


def make_digest(c):
    """Per-iteration digest of the compiled reference over a whole run."""
    x, y = instances.uniform_instance(c["n"], seed=c["seed"])
    d = oracle.distances(x, y)
    ref = oracle.Ref(digest_params(c), d)
    ref.initialize()
    h = b""
    out = dict(c, iter_best=[], glob_best=[], digests={})
    for it in range(1, c["iters"] + 1):
        ref.iterate()
        h = chain_digest(h, ref.tours(), ref.lengths(), ref.pheromone())
        out["iter_best"].append(int(ref.iter_best()))
        out["glob_best"].append(int(ref.glob_best()))
        if it in c["checkpoints"]:
            out["digests"][str(it)] = h.hex()
    out["best_tour"] = [int(v) for v in ref.best_tour()]
    ref.close()
    return out


def main():
    index = {}
    for c in CASES:
        arrays, meta = make_case(c)
        np.savez_compressed(os.path.join(HERE, c["name"] + ".npz"), **arrays)
        index[c["name"]] = meta
        print(c["name"], "glob_best", arrays["glob_best"][-1])
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(index, f, indent=1)
    dg = make_digest(DIGEST)
    with open(os.path.join(HERE, DIGEST["name"] + ".json"), "w") as f:
        json.dump(dg, f)
    print(DIGEST["name"], "glob_best", dg["glob_best"][-1])


if __name__ == "__main__":
    main()
