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


def main():
    index = {}
    for c in CASES:
        arrays, meta = make_case(c)
        np.savez_compressed(os.path.join(HERE, c["name"] + ".npz"), **arrays)
        index[c["name"]] = meta
        print(c["name"], "glob_best", arrays["glob_best"][-1])
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()
