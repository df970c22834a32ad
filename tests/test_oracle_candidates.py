"""An independent check of the oracle's candidate-list construction (k < n,
the engine's extension: the reference has full rows only) against a direct
Python restatement of the rule, on small instances: the roulette over the k
candidates of the current city in candidate order (a sequential float32
sum; the walk of src/Colony.cu:833-846), and the best-choice fallback (the
unvisited city with the largest choice value, lowest index on ties) when the
sum is 0 or the walk runs past the row.  Noaging Ant System, no prior, so the
candidate weight is the choice value."""
import numpy as np
import pytest

import oracle
from acogpu_gb300 import _abi, rng
from helpers import instance, params

F32 = np.float32


def restated_tours(choice, nn, k, m, seed, iteration):
    n = choice.shape[0]
    tours = np.zeros((m, n), np.int32)
    for ant in range(m):
        u0 = rng.uniform(seed, iteration, ant, 0)
        start = int(F32(u0) * F32(n))
        vis = np.zeros(n, bool)
        vis[start] = True
        t = [start]
        for x in range(1, n):
            cur = t[-1]
            row = nn[cur, :k]
            w = [F32(0) if vis[c] else F32(choice[cur, c]) for c in row]
            s = F32(0)
            for v in w:
                s = F32(s + v)
            nxt = None
            if s > 0:
                rnd = F32(F32(rng.uniform(seed, iteration, ant, x)) * s)
                i, partial = 0, w[0]
                while partial <= rnd:
                    i += 1
                    if i >= k:
                        i = -1
                        break
                    partial = F32(partial + w[i])
                if i >= 0:
                    nxt = int(row[i])
            if nxt is None:  # best choice among the unvisited, lowest index on ties
                best, bv = -1, F32(-1)
                for j in range(n):
                    if not vis[j] and F32(choice[cur, j]) > bv:
                        best, bv = j, F32(choice[cur, j])
                nxt = best
            vis[nxt] = True
            t.append(nxt)
        tours[ant] = t
    return tours


@pytest.mark.parametrize("n,k,seed", [(30, 3, 1), (40, 8, 2), (25, 5, 3), (36, 1, 4)])
def test_candidate_construction_matches_restatement(n, k, seed):
    _, _, d = instance(n, seed, kind="clustered" if seed % 2 else "uniform")
    p = params(num_ants=6, beta=2.0, rho=0.3, cand_k=k, seed=100 + seed,
               nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
               fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO)
    q = oracle.Port(p, d, threads=1)
    q.initialize()
    nn = q.nn()
    for it in range(3):
        choice = q.choice().copy()
        expect = restated_tours(choice, nn, k, p.num_ants, p.seed, it)
        q.iterate()
        assert np.array_equal(q.tours(), expect), it
    q.close()
