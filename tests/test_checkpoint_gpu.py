"""GPU tests of checkpoint / resume (aco_colony_save / _load): a colony
loaded from a checkpoint continues bit for bit as the saved one, in both
deposit orders, with aging and with a learned prior; loads into another
instance or configuration, and damaged files, are refused."""
import numpy as np
import pytest

import acogpu_gb300 as aco
from acogpu_gb300 import _abi
from acogpu_gb300.colony import AcoError
from helpers import instance

pytestmark = pytest.mark.gpu

FAST = dict(nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO)


def make(d, p):
    c = aco.Colony(d, params=p, num_ants=p.num_ants)
    c.initialize()
    return c


def same(a, b, aging, ctx):
    assert np.array_equal(a.tours(), b.tours()), ctx
    assert np.array_equal(a.tour_lengths(), b.tour_lengths()), ctx
    assert np.array_equal(a.pheromone().view(np.uint32), b.pheromone().view(np.uint32)), ctx
    assert np.array_equal(a.choice_info().view(np.uint32), b.choice_info().view(np.uint32)), ctx
    assert a.getIterBestDist() == b.getIterBestDist(), ctx
    assert a.getGlobBestDist() == b.getGlobBestDist(), ctx
    assert np.array_equal(a.best_tour(), b.best_tour()), ctx
    if aging:
        sa, sb = a.aging_state(), b.aging_state()
        for k in sa:
            assert np.array_equal(np.asarray(sa[k]), np.asarray(sb[k])), (ctx, k)


@pytest.mark.parametrize("variant,aging,deposit", [
    (_abi.ACO_ANT_SYSTEM, 0, _abi.ACO_DEPOSIT_DETERMINISTIC),
    (_abi.ACO_RANK_BASED, 1, _abi.ACO_DEPOSIT_DETERMINISTIC),
    (_abi.ACO_ANT_SYSTEM, 0, _abi.ACO_DEPOSIT_ATOMIC),
])
def test_resume_continues_bit_for_bit(tmp_path, variant, aging, deposit):
    _, _, d = instance(180, 44, kind="clustered")
    p = _abi.default_params(num_ants=60, variant=variant, rank_w=6, aging=aging, cand_k=24,
                            beta=2.0, rho=0.2, seed=44, deposit=deposit, **FAST)
    if aging:
        (p.min_retirement_age, p.max_retirement_age, p.global_performance,
         p.min_population_limit) = (3, 6, 2, 40)
    a = make(d, p)
    a.run(7)
    a.synchronize()
    path = tmp_path / "colony.ckpt"
    a.save(path)
    b = make(d, p)
    b.constructSolution()  # some unrelated progress, overwritten by the load
    b.load(path)
    same(a, b, aging, "right after load")
    if deposit == _abi.ACO_DEPOSIT_ATOMIC:
        # atomic adds are order-free, so two colonies part in the last bits
        # after any iteration; the restored state itself is exact (above)
        a.constructSolution()
        b.constructSolution()
        assert np.allclose(a.pheromone(), b.pheromone(), rtol=1e-5, atol=0)
        a.close()
        b.close()
        return
    for it in range(6):
        a.constructSolution()
        b.constructSolution()
        same(a, b, aging, f"iteration {it} after resume")
    b.run(3)
    a.run(3)
    a.synchronize()
    b.synchronize()
    same(a, b, aging, "graph replay after resume")
    a.close()
    b.close()


def test_resume_keeps_a_learned_prior(tmp_path):
    from acogpu_gb300.prior import EdgePrior
    from acogpu_gb300 import instances
    x, y = instances.uniform_instance(150, seed=3)
    p = _abi.default_params(num_ants=40, cand_k=20, beta=2.0, rho=0.2, seed=3, **FAST)
    a = aco.Colony(coords=(x, y), params=p, num_ants=40)
    a.initialize()
    EdgePrior(seed=5).apply(a, floor=0.05)
    a.run(4)
    a.synchronize()
    a.save(tmp_path / "p.ckpt")
    b = aco.Colony(coords=(x, y), params=p, num_ants=40)
    b.initialize()  # plain heuristic; the checkpoint carries the prior's
    b.load(tmp_path / "p.ckpt")
    for _ in range(3):
        a.constructSolution()
        b.constructSolution()
    same(a, b, False, "prior resume")


def test_refused_loads(tmp_path):
    _, _, d = instance(90, 7)
    p = _abi.default_params(num_ants=20, cand_k=16, beta=2.0, rho=0.2, seed=7, **FAST)
    a = make(d, p)
    a.run(2)
    a.synchronize()
    path = tmp_path / "a.ckpt"
    a.save(path)
    _, _, d2 = instance(90, 8)
    other_instance = make(d2, p)
    with pytest.raises(AcoError) as e:
        other_instance.load(path)
    assert e.value.status == _abi.ACO_ERR_INVALID_ARGUMENT
    q = _abi.AcoParams.from_buffer_copy(p)
    q.rho = 0.3
    other_params = make(d, q)
    with pytest.raises(AcoError) as e:
        other_params.load(path)
    assert e.value.status == _abi.ACO_ERR_INVALID_ARGUMENT
    data = open(path, "rb").read()
    (tmp_path / "short.ckpt").write_bytes(data[: len(data) // 2])
    with pytest.raises(AcoError) as e:
        make(d, p).load(tmp_path / "short.ckpt")
    assert e.value.status == _abi.ACO_ERR_FORMAT
    (tmp_path / "junk.ckpt").write_bytes(b"\0" * 4096)
    with pytest.raises(AcoError) as e:
        make(d, p).load(tmp_path / "junk.ckpt")
    assert e.value.status == _abi.ACO_ERR_FORMAT
    with pytest.raises(AcoError) as e:
        make(d, p).load(tmp_path / "absent.ckpt")
    assert e.value.status == _abi.ACO_ERR_IO
