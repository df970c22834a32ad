"""Throughput benchmark of the GB300 ACO engine.

Default workload (`--workload parity_batch8`; one "step" = one full
iteration of the hot path for every instance of the batch: construction of
every ant's tour, tour lengths and bests, evaporation + deposit, next
choice-info): the reference's own algorithm -- the Ant System with ant
aging, full-row roulette over the whole nn row in the order of its CPU
quicksort, the libm heuristic, select_local_best as the fallback, tau0 =
1e-6, the sequential (deterministic) deposit -- on a batch of 8 instances of
n = 1000 cities drawn from 20 Gaussian clusters (sigma 300) in
[0,10000)^2, m = 1000 ants each, rho = 0.1, beta = 2.  Seeded synthetic
instances (no TSPLIB file is read).  Before the timed steps the integer tour
lengths of the first iterations of every instance are compared bit for bit
with the CPU restatement of the reference path, and the result is printed
in the line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload parity_batch8|rbas_aging_n1000|batch512|large4096|learned]

Prints one JSON line (rank 0).  `value` is tours/s over the device-timed
steps (CUDA events on the batch's stream; the batch's working set, about
370 MB, is larger than L2); `e2e` is the same metric through the public API
from host buffers (create from host coordinates, initialize, per step one
iteration and a read of every instance's best length).  `--impl reference`
times the reference's CPU algorithm (its restatement in C, all host
threads) on the identical configuration.  With --gpus N > 1 every rank runs
its own batch of 8 instances (weak scaling; no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from acogpu_gb300 import distrib  # noqa: E402  (pure Python: no library load)

N_CITIES, N_ANTS, RANK_W, CAND_K, RHO, BETA = 1000, 1000, 6, 30, 0.1, 2.0
INSTANCE_SEED = 2026
WORKLOAD = ("rank-based Ant System with aging, n=1000 (20 Gaussian clusters, sigma 300, "
            "[0,10000)^2), m=1000, w=6, k=30, rho=0.1")
L2_FLUSH_BYTES = 256 << 20
REF_BUDGET_S = 60.0  # CPU time the reference arm spends on its timed sample
# Default timed steps per workload: about a second of timed work for the
# single-colony lines (clock samples every 200 ms fall inside it).
DEFAULT_STEPS = {"parity_batch8": 40, "rbas_aging_n1000": 2000, "large4096": 300,
                 "batch512": 10, "learned": 0}
# Parity-mode batch: the reference's own algorithm on 8 clustered n = 1000
# instances (see the module docstring).
PARITY_COUNT, PARITY_N, PARITY_SEED0 = 8, 1000, 2026
PARITY_CHECK_ITERS = 2  # iterations of every instance checked against the port before timing
PARITY_WORKLOAD = ("reference algorithm (Ant System with aging, full-row roulette in the "
                   "reference nn order, libm heuristic, select_local_best fallback, tau0 1e-6, "
                   "sequential deposit), batch of 8 instances of n=1000 (20 Gaussian clusters, "
                   "sigma 300, [0,10000)^2), m=1000 each, rho=0.1, beta=2")
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parity_params():
    """The reference's own configuration (AntSystem with aging,
    src/AntSystem.cu:160-182; defaults inc/default.h) in parity mode."""
    from acogpu_gb300 import _abi
    return _abi.default_params(
        num_ants=PARITY_N, variant=_abi.ACO_ANT_SYSTEM, aging=1, cand_k=0, rho=RHO, beta=BETA,
        nn_order=_abi.ACO_NN_REFERENCE_QSORT, heuristic=_abi.ACO_HEURISTIC_LIBM,
        fallback=_abi.ACO_FALLBACK_REFERENCE, tau0_mode=_abi.ACO_TAU0_REFERENCE,
        deposit=_abi.ACO_DEPOSIT_DETERMINISTIC, seed=1234)


def parity_instances(rank=0):
    from acogpu_gb300 import instances
    return [instances.clustered_instance(PARITY_N, seed=PARITY_SEED0 + 100 * rank + i)
            for i in range(PARITY_COUNT)]


def parity_config():
    """The config dict of both arms (identical, so the two lines compare)."""
    return {"workload": PARITY_WORKLOAD, "instances": PARITY_COUNT, "n": PARITY_N,
            "m": PARITY_N, "k": PARITY_N, "variant": "AS", "aging": True, "rho": RHO,
            "beta": BETA, "nn_order": "reference quicksort", "heuristic": "libm powf",
            "fallback": "select_local_best", "tau0": 1e-6, "deposit": "sequential",
            "iterations_per_step": 1}


def instance_params(p, i):
    """Parameters of instance i of a batch (aco_batch_create: seed + i * golden)."""
    from acogpu_gb300 import _abi
    q = _abi.AcoParams.from_buffer_copy(p)
    q.seed = (p.seed + i * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    return q


def workload_params():
    from acogpu_gb300 import _abi
    return _abi.default_params(
        num_ants=N_ANTS, variant=_abi.ACO_RANK_BASED, rank_w=RANK_W, aging=1, cand_k=CAND_K,
        rho=RHO, beta=BETA, nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
        fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO,
        deposit=_abi.ACO_DEPOSIT_DETERMINISTIC, seed=1234)


def workload_instance():
    from acogpu_gb300 import instances
    x, y = instances.clustered_instance(N_CITIES, seed=INSTANCE_SEED)
    return x, y, instances.euc2d_distances(x, y)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={CLOCK_FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [v.strip() for v in line.split(",")]
                if len(f) >= 9 and f[1].isdigit():
                    rows.append(f)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [int(r[1]) for r in rows]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = [nm for i, nm in enumerate(names) if any(r[5 + i] == "Active" for r in rows)]
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]),
                "samples": len(rows), "reasons": reasons}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def profiled_traffic(name="construct_staged_rbas_aging_n1000.md", key="traffic_bytes_per_launch"):
    """DRAM bytes per launch of the construction kernel, from the committed
    ncu summary (dram__bytes_read.sum + dram__bytes_write.sum of one capture)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def construct_bytes(n, k, tours, fallbacks):
    """Algorithmic bytes of the construction kernel: per ant-step the k
    candidate ids and k choice weights (8k), the tour write and the distance
    lookup (8); per fallback step one full choice row (4n)."""
    return tours * (n - 1) * (8 * k + 8) + fallbacks * 4 * n


def cpu_baseline(steps_iters=2):
    """The CPU oracle on this host's cores, same algorithm and instance as
    the GPU run, a bounded sample of iterations."""
    import oracle
    x, y, d = workload_instance()
    threads = os.cpu_count() or 1
    q = oracle.Port(workload_params(), d, threads=threads)
    q.initialize()
    q.iterate(1)
    t0 = time.perf_counter()
    q.iterate(steps_iters)
    dt = time.perf_counter() - t0
    tours = steps_iters * q.num_valid()
    q.close()
    return {"value": tours / dt, "unit": "tours/s", "cores": threads, "kind": "port",
            "sample": f"{steps_iters} iterations of the same workload (after 1 warm-up) with the "
                      f"C oracle, construction spread over {threads} threads"}


def run_reference(args, rank):
    """Reference arm: the reference's CPU algorithm (full-row roulette, its
    only construction rule; AS update, its rank-based update is an empty
    stub), restated in C, on the host cores, same instance and ant count."""
    if rank != 0:
        return None
    import oracle
    from acogpu_gb300 import _abi
    x, y, d = workload_instance()
    p = _abi.default_params(num_ants=N_ANTS, aging=1, rho=RHO, beta=BETA, cand_k=0,
                            nn_order=_abi.ACO_NN_REFERENCE_QSORT,
                            heuristic=_abi.ACO_HEURISTIC_LIBM,
                            fallback=_abi.ACO_FALLBACK_REFERENCE, seed=1234)
    threads = os.cpu_count() or 1
    q = oracle.Port(p, d, threads=threads)
    q.initialize()
    for _ in range(args.warmup):
        q.iterate()
    # A bounded sample of the requested steps: about REF_BUDGET_S seconds of
    # CPU work (the rate, not the count, is the result).
    tours, done = 0, 0
    t0 = time.perf_counter()
    while done < args.steps:
        q.iterate()
        tours += q.num_valid()
        done += 1
        if time.perf_counter() - t0 > REF_BUDGET_S:
            break
    dt = time.perf_counter() - t0
    v = tours / dt
    return {"metric": "tours/s", "value": v, "unit": "tours/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / done, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD + " -- reference CPU algorithm: full-row roulette "
                       "(no candidate lists), AS update (the reference's rank-based update is an "
                       "empty stub)", "n": N_CITIES, "m": N_ANTS, "k": N_CITIES},
            "cpu_baseline": {"value": v, "unit": "tours/s", "cores": threads, "kind": "port",
                             "sample": f"{done} of {args.steps} iterations (at most "
                                       f"{REF_BUDGET_S:.0f} s) after {args.warmup} warm-up, "
                                       f"C restatement of the reference CPU path, {threads} "
                                       f"threads"},
            "e2e": {"value": v, "unit": "tours/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def run_ours(args, rank, world, local):
    import torch
    import acogpu_gb300 as aco

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    x, y, d = workload_instance()
    p = workload_params()
    p.seed = distrib.replica_seed(1234, rank)  # independent replicas

    # The colony's own stream (not the legacy default stream, which cannot be
    # captured): an iteration is one replay of the captured graph.
    stream = torch.cuda.Stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---------------- device-timed steps
    col = aco.Colony(d, params=p, num_ants=N_ANTS)
    col.set_stream(stream.cuda_stream)
    col.initialize()
    for _ in range(args.warmup):
        col.constructSolution()
    col.synchronize()
    st0 = col.stats()
    launches0 = col.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    stage = np.zeros(6)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk, torch.cuda.stream(stream):
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()  # L2 flush, outside the timed events
            ev[i][0].record(stream)
            col.constructSolution()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_s = sum(step_ms) / 1e3
    st1 = col.stats()
    launches = col.launch_count() - launches0
    tours = st1["tours_built"] - st0["tours_built"]
    fallbacks = st1["fallbacks"] - st0["fallbacks"]
    # Stage breakdown: further iterations with per-stage events (outside the
    # timed steps above), L2 flushed before each.
    stage_steps = min(args.steps, 20)
    with torch.cuda.stream(stream):
        for _ in range(stage_steps):
            flush.zero_()
            stage += col.constructSolution(timers=True)
    stage *= args.steps / max(1, stage_steps)
    col.close()

    # ---------------- end to end through the public API (host buffers)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    e = aco.Colony(d, params=p, num_ants=N_ANTS)
    e.initialize()
    d2h = 0
    for _ in range(args.steps):
        e.constructSolution()
        e.getIterBestDist()
        e.getGlobBestDist()
        e.getNumValidAnts()
        d2h += 3 * 96  # three state reads (the device state block, padded)
    tour = e.getTour()
    d2h += 4 * N_CITIES
    e_stats = e.stats()
    torch.cuda.synchronize()
    e_wall = time.perf_counter() - t0
    e.close()
    barrier()
    e_tours = e_stats["tours_built"]

    # max over ranks of the times, sum of the work
    (dev_s, e_wall, wall), (tours_all, e_tours_all) = distrib.reduce_times_and_counts(
        [dev_s, e_wall, wall], [tours, e_tours], device=dev)
    if rank != 0:
        return None

    pk = peaks()
    hbm = pk.get("hbm_gbs")
    construct_s = stage[1] / 1e3
    bytes_c = construct_bytes(N_CITIES, CAND_K, tours, fallbacks)
    achieved = bytes_c / construct_s / 1e9
    return {
        "metric": "tours/s", "value": tours_all / dev_s, "unit": "tours/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "wall_ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": N_CITIES, "m": N_ANTS, "k": CAND_K, "w": RANK_W,
                   "rho": RHO, "beta": BETA, "aging": True, "deposit": "deterministic",
                   "iterations_per_step": 1,
                   "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MB write, untimed)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "ant_steps_per_s": tours_all * (N_CITIES - 1) / dev_s,
        "stage_ms_per_step": {"construct": stage[1] / args.steps,
                              "epilogue": stage[2] / args.steps,
                              "pheromone": stage[4] / args.steps},
        "fallback_rate": fallbacks / max(1, tours * (N_CITIES - 1)),
        "gpu_launches": int(launches) * world,
        "roofline": {"bound": "hbm", "kernel": "k_construct_staged", "achieved": achieved,
                     "peak": hbm, "unit": "GB/s", "frac": achieved / hbm if hbm else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if hbm else None,
                     "algorithmic_bytes_per_launch": bytes_c / args.steps,
                     "traffic": profiled_traffic(),
                     "traffic_source": "profiles/construct_staged_rbas_aging_n1000.md (ncu)"},
        "e2e": {"value": e_tours_all / e_wall, "unit": "tours/s",
                "h2d_bytes_per_step": 4 * N_CITIES * N_CITIES / args.steps,
                "d2h_bytes_per_step": d2h / args.steps, "tour_head": tour[:24]},
        "clocks": clk.summary(),
    }


def parity_check(batch, insts, p, iters):
    """Runs `iters` iterations of a fresh batch and of the CPU restatement of
    the reference path on every instance; returns (all integer tour lengths
    equal, tours compared)."""
    import oracle
    from acogpu_gb300 import instances
    ports = []
    for i, (x, y) in enumerate(insts):
        q = oracle.Port(instance_params(p, i), instances.euc2d_distances(x, y),
                        threads=os.cpu_count() or 1)
        q.initialize()
        ports.append(q)
    same, compared = True, 0
    for _ in range(iters):
        batch.run(1)
        batch.synchronize()
        for i, q in enumerate(ports):
            q.iterate()
            g = batch.colony(i).tour_lengths()
            same = same and bool(np.array_equal(g, q.lengths()))
            compared += int(q.num_valid())
    for q in ports:
        q.close()
    return same, compared


def rows_bytes(n, tours):
    """Algorithmic bytes of the long-row construction: per ant-step one
    candidate row staged (n choice values and n int16 ids) and the tour
    write."""
    return tours * (n - 1) * (6 * n + 4)


def run_parity(args, rank, world, local):
    """The parity-mode batch (the reference's own algorithm), device-timed and
    end to end; 8 instances per GPU (weak scaling)."""
    import torch
    import acogpu_gb300 as aco
    torch.cuda.set_device(local)
    insts = parity_instances(rank)
    p = parity_params()
    p.seed = distrib.replica_seed(1234, rank)
    # ---- bit-exact check of the first iterations against the CPU path
    b = aco.Batch(insts, params=p, num_ants=PARITY_N)
    b.initialize()
    checked, compared = parity_check(b, insts, p, PARITY_CHECK_ITERS) if rank == 0 else (None, 0)
    b.run(max(0, args.warmup - PARITY_CHECK_ITERS))
    b.synchronize()
    built0, launches0 = b.tours_built(), b.launch_count()
    fb0 = sum(b.colony(i).stats()["fallbacks"] for i in range(len(insts)))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            ev[i][0].record()
            b.run(1)
            b.synchronize()
            ev[i][1].record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    dev_s = sum(a.elapsed_time(e) for a, e in ev) / 1e3
    tours = b.tours_built() - built0
    launches = b.launch_count() - launches0
    fallbacks = sum(b.colony(i).stats()["fallbacks"] for i in range(len(insts))) - fb0
    # Construction alone, event-timed on the batch's stream by the library
    # (the autotuner's timing runs reset the instances afterwards).
    tune = b.autotune()
    b.close()
    # ---- end to end through the public API, host buffers
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e = aco.Batch(insts, params=p, num_ants=PARITY_N)
    t_create = time.perf_counter() - t0
    e.initialize()
    t_setup = time.perf_counter() - t0
    d2h = 0
    for _ in range(args.steps):
        e.run(1)
        e.glob_best()
        d2h += 8 * len(insts)
    e_built = e.tours_built()
    e.synchronize()
    e_wall = time.perf_counter() - t0
    e.close()
    (dev_s, e_wall), (tours_all, e_tours_all, launches) = distrib.reduce_times_and_counts(
        [dev_s, e_wall], [tours, e_built, launches], device=torch.device("cuda", local))
    if rank != 0:
        return None
    hbm = peaks().get("hbm_gbs")
    per_launch = rows_bytes(PARITY_N, tours / args.steps)
    construct_s = tune["construct_ms"] / 1e3
    achieved = per_launch / construct_s / 1e9 if construct_s > 0 else None
    return {
        "metric": "tours/s", "value": tours_all / dev_s, "unit": "tours/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(parity_config(),
                       l2="working set about 370 MB per GPU, larger than L2"),
        "same_config": True,  # --impl reference runs this exact config and metric
        "ant_steps_per_s": tours_all * (PARITY_N - 1) / dev_s,
        "parity": {"integer_tour_lengths_bit_exact": checked,
                   "iterations_checked_per_instance": PARITY_CHECK_ITERS,
                   "tours_compared": compared,
                   "against": "C restatement of the reference CPU path (oracle/aco_oracle.c)"},
        "fallback_rate": fallbacks / max(1, tours * (PARITY_N - 1)),
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_batch_construct_rows", "achieved": achieved,
                     "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if (hbm and achieved) else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if hbm else None,
                     "algorithmic_bytes_per_launch": per_launch,
                     "construct_ms": tune["construct_ms"],
                     "traffic": profiled_traffic("construct_rows_parity_batch8.md"),
                     "traffic_source": "profiles/construct_rows_parity_batch8.md (ncu)"},
        "e2e": {"value": e_tours_all / e_wall, "unit": "tours/s",
                "h2d_bytes_per_step": 8 * PARITY_N * PARITY_COUNT / args.steps,
                "d2h_bytes_per_step": d2h / args.steps, "create_s": t_create,
                "setup_s": t_setup},
        "clocks": clk.summary(),
    }


def parity_cpu_baseline(threads=None, iters=1):
    """The CPU restatement on this host's cores: one instance of the batch, a
    bounded sample of iterations."""
    import oracle
    from acogpu_gb300 import instances
    threads = threads or os.cpu_count() or 1
    x, y = parity_instances(0)[0]
    q = oracle.Port(instance_params(parity_params(), 0), instances.euc2d_distances(x, y),
                    threads=threads)
    q.initialize()
    t0 = time.perf_counter()
    q.iterate(iters)
    dt = time.perf_counter() - t0
    tours = iters * q.num_valid()
    q.close()
    return {"value": tours / dt, "unit": "tours/s", "cores": threads, "kind": "port",
            "sample": f"{iters} iteration(s) of instance 0 of the batch (from its start), "
                      f"construction spread over {threads} threads"}


def run_reference_parity(args, rank):
    """Reference arm on the parity workload: the reference CPU algorithm (its
    restatement in C) on the same 8 instances, all host threads; a bounded
    sample of iterations, round-robin over the instances."""
    if rank != 0:
        return None
    import oracle
    from acogpu_gb300 import instances
    threads = os.cpu_count() or 1
    insts = parity_instances(0)
    p = parity_params()
    ports = []
    for i, (x, y) in enumerate(insts):
        q = oracle.Port(instance_params(p, i), instances.euc2d_distances(x, y), threads=threads)
        q.initialize()
        ports.append(q)
    for w in range(args.warmup):
        ports[w % len(ports)].iterate()
    tours, done = 0, 0
    t0 = time.perf_counter()
    while done < args.steps * len(ports):
        q = ports[done % len(ports)]
        q.iterate()
        tours += q.num_valid()
        done += 1
        if time.perf_counter() - t0 > REF_BUDGET_S:
            break
    dt = time.perf_counter() - t0
    for q in ports:
        q.close()
    v = tours / dt
    # The reference itself is single-threaded: the same algorithm on one core
    # (one iteration of instance 0, after one untimed iteration), for scale.
    x0, y0 = insts[0]
    q1 = oracle.Port(instance_params(p, 0), instances.euc2d_distances(x0, y0), threads=1)
    q1.initialize()
    q1.iterate()
    t1 = time.perf_counter()
    q1.iterate()
    v1 = q1.num_valid() / (time.perf_counter() - t1)
    q1.close()
    return {"metric": "tours/s", "value": v, "unit": "tours/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt * len(ports) / max(1, done), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(parity_config(),
                           l2="working set about 370 MB per GPU, larger than L2"),
            "same_config": True,
            "cpu_baseline": {"value": v, "unit": "tours/s", "cores": threads, "kind": "port",
                             "sample": f"{done} instance-iterations of the {args.steps} x "
                                       f"{len(ports)} requested (at most {REF_BUDGET_S:.0f} s), "
                                       f"after {args.warmup} warm-up, C restatement of the "
                                       f"reference CPU path, {threads} threads"},
            "e2e": {"value": v, "unit": "tours/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "single_core": {"value": v1, "unit": "tours/s", "cores": 1,
                            "sample": "iteration 2 of instance 0, C restatement, 1 thread"}}


BATCH_COUNT, BATCH_CAP, BATCH_K = 512, 1024, 20
LEARN_CHUNK = 2048  # training instances labelled per batch
BATCH_WORKLOAD = ("512 instances, n log-uniform in [50,2000] (uniform and clustered alternating), "
                  "m = min(n, 1024), k=20, AS, rho=0.1, beta=2; one persistent construction "
                  "launch per iteration over a work queue, graph-replayed, autotuned")


def batch_instances(count=BATCH_COUNT):
    from acogpu_gb300 import instances
    sizes = instances.batch_sizes(count, seed=7)
    out = []
    for i, n in enumerate(sizes):
        gen = instances.uniform_instance if i % 2 == 0 else instances.clustered_instance
        out.append(gen(int(n), seed=10_000 + i))
    return out


def batch_params():
    from acogpu_gb300 import _abi
    return _abi.default_params(num_ants=BATCH_CAP, cand_k=BATCH_K, rho=RHO, beta=BETA,
                               nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                               fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO,
                               seed=4321)


def batch_cpu_sample(iters=2, per_stratum=2, strata=8, budget_s=REF_BUDGET_S):
    """The uneven batch on the CPU restatement, all host threads: a stratified
    sample of instances (per_stratum from each of `strata` size bands), `iters`
    iterations each after one warm-up, extrapolated to the whole batch by the
    ant-steps it holds (sum of m (n - 1): with candidate lists a step costs
    about the same at every n).  Returns (tours/s, description)."""
    import oracle
    from acogpu_gb300 import instances
    threads = os.cpu_count() or 1
    insts = batch_instances()
    sizes = np.array([len(x) for x, _ in insts])
    ants = np.minimum(sizes, BATCH_CAP)
    order = np.argsort(sizes, kind="stable")
    bands = np.array_split(order, strata)
    picked = [int(b[(len(b) - 1) * j // max(1, per_stratum - 1)]) for b in bands
              for j in range(per_stratum)]
    t_s, steps_s = 0.0, 0.0
    t_start = time.perf_counter()
    for i in picked:
        x, y = insts[i]
        pi = instance_params(batch_params(), i)
        pi.num_ants = int(ants[i])
        q = oracle.Port(pi, instances.euc2d_distances(x, y), threads=threads)
        q.initialize()
        q.iterate(1)
        t0 = time.perf_counter()
        q.iterate(iters)
        t_s += time.perf_counter() - t0
        steps_s += iters * float(ants[i]) * (sizes[i] - 1)
        q.close()
        if time.perf_counter() - t_start > budget_s:
            break
    total_steps = float((ants * (sizes - 1)).sum())
    t_batch = t_s / steps_s * total_steps  # seconds for one whole-batch iteration
    v = float(ants.sum()) / t_batch
    desc = (f"{len(picked)} of {len(insts)} instances (stratified by size, {per_stratum} from each "
            f"of {strata} bands), {iters} iterations each after 1 warm-up, extrapolated to the "
            f"whole batch by its ant-steps (sum of m(n-1)); C restatement, {threads} threads")
    return v, threads, desc


def run_reference_batch(args, rank):
    """Reference arm on the uneven batch: the same rule (candidate lists of
    20, best-choice fallback -- the reference itself has no candidate lists)
    on the CPU restatement, from a stratified sample."""
    if rank != 0:
        return None
    v, threads, desc = batch_cpu_sample()
    return {"metric": "tours/s", "value": v, "unit": "tours/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": batch_config(BATCH_COUNT),
            "cpu_baseline": {"value": v, "unit": "tours/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": v, "unit": "tours/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def batch_config(count):
    sizes = np.array([len(x) for x, _ in batch_instances(count)])
    return {"workload": BATCH_WORKLOAD, "instances": int(count),
            "cities_total": int(sizes.sum()),
            "ants_per_iteration": int(np.minimum(sizes, BATCH_CAP).sum()),
            "l2": "working set 5+ GB, larger than L2"}


def run_batch(args, rank, world, local):
    """Batched uneven instances: whole-batch iterations, device-timed.  On N
    GPUs, 512·N instances are generated and sharded by estimated cost (weak
    scaling, no collective on the data path)."""
    import torch
    import acogpu_gb300 as aco
    torch.cuda.set_device(local)
    allinst = batch_instances(args.batch_instances * world)
    sizes_all = [len(x) for x, _ in allinst]
    mine = distrib.shard_instances(sizes_all, np.minimum(sizes_all, BATCH_CAP), BATCH_K,
                                   world)[rank]
    insts = [allinst[i] for i in mine]
    p = batch_params()
    p.seed = distrib.replica_seed(4321, rank)
    t0 = time.perf_counter()
    b = aco.Batch(insts, params=p, num_ants=BATCH_CAP)
    b.initialize()
    tune = b.autotune()
    setup_s = time.perf_counter() - t0
    b.run(args.warmup)
    b.synchronize()
    built0, launches0 = b.tours_built(), b.launch_count()
    fb0 = np.array([b.colony(i).stats()["fallbacks"] for i in range(len(insts))], np.float64)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record()
        b.run(args.steps)
        b.synchronize()
        end.record()
        torch.cuda.synchronize()
    dev_s = start.elapsed_time(end) / 1e3
    tours = b.tours_built() - built0
    launches = b.launch_count() - launches0
    sizes = np.array([len(x) for x, _ in allinst])
    ants = np.minimum(sizes, BATCH_CAP)
    # Roofline of the construction kernel on this GPU's shard: the bytes of
    # construct_bytes per instance (its fallbacks counted over the timed
    # steps) over the autotuner's event-timed construction launch.
    fb1 = np.array([b.colony(i).stats()["fallbacks"] for i in range(len(insts))], np.float64)
    my_n = np.array([len(x) for x, _ in insts], np.float64)
    my_m = np.minimum(my_n, BATCH_CAP)
    my_k = np.minimum(BATCH_K, my_n - 1)
    bytes_c = float((my_m * (my_n - 1) * (8 * my_k + 8)).sum() +
                    ((fb1 - fb0) / args.steps * 4 * my_n).sum())
    hbm = peaks().get("hbm_gbs")
    achieved = bytes_c / (tune["construct_ms"] / 1e3) / 1e9
    # DRAM traffic: the 32-instance capture's bytes per ant-step times this
    # shard's ant-steps (the whole batch does not fit an ncu capture).
    t32 = profiled_traffic("construct_batch_uneven32.md")
    s32 = profiled_traffic("construct_batch_uneven32.md", "ant_steps_per_launch")
    batch_traffic = (t32 / s32 * float((my_m * (my_n - 1)).sum())) if (t32 and s32) else None
    best = b.glob_best()
    b.close()
    (dev_s,), (tours, launches, best_sum) = distrib.reduce_times_and_counts(
        [dev_s], [tours, launches, float(best.sum())], device=torch.device("cuda", local))
    if rank != 0:
        return None
    return {"metric": "tours/s", "value": tours / dev_s, "unit": "tours/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": batch_config(len(allinst)),
            "ant_steps_per_s": float((ants * (sizes - 1)).sum()) * args.steps / dev_s,
            "autotune": tune, "setup_s": setup_s, "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "k_batch_construct", "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm if hbm else None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if hbm else None,
                         "algorithmic_bytes_per_launch": bytes_c, "traffic": batch_traffic,
                         "traffic_source": "profiles/construct_batch_uneven32.md (ncu of one "
                                           "launch over a 32-instance slice), scaled by ant-steps"},
            "mean_best_length": best_sum / len(allinst), "clocks": clk.summary()}


def run_large(args, rank, world, local):
    """Large single instance: n=4096 uniform in [0,100000)^2, m=512, k=32,
    atomic deposit, plain AS (the cluster construction kernel)."""
    import torch
    import acogpu_gb300 as aco
    from acogpu_gb300 import _abi, instances
    torch.cuda.set_device(local)
    x, y = instances.uniform_instance(4096, box=100000, seed=4096)
    p = _abi.default_params(num_ants=512, cand_k=32, rho=RHO, beta=BETA,
                            nn_order=_abi.ACO_NN_STABLE, heuristic=_abi.ACO_HEURISTIC_DEVICE,
                            fallback=_abi.ACO_FALLBACK_BEST, tau0_mode=_abi.ACO_TAU0_DORIGO,
                            deposit=_abi.ACO_DEPOSIT_ATOMIC, seed=77 + rank)
    col = aco.Colony(coords=(x, y), params=p, num_ants=512)
    col.initialize()
    for _ in range(args.warmup):
        col.constructSolution()
    col.synchronize()
    st0, l0 = col.stats(), col.launch_count()
    stage = np.zeros(6)
    ms = 0.0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t = col.constructSolution(timers=True)
            stage += t
            ms += float(t.sum())
    st1 = col.stats()
    tours = st1["tours_built"] - st0["tours_built"]
    fallbacks = st1["fallbacks"] - st0["fallbacks"]
    bytes_c = construct_bytes(4096, 32, tours, fallbacks)
    hbm = peaks().get("hbm_gbs")
    achieved = bytes_c / (stage[1] / 1e3) / 1e9
    best = col.getGlobBestDist()
    launches = col.launch_count() - l0
    col.close()
    # N GPUs run independent replicas: the slowest rank's time, every rank's tours
    (ms,), (tours_all,) = distrib.reduce_times_and_counts(
        [ms], [tours], device=torch.device("cuda", local))
    if rank != 0:
        return None
    return {"metric": "tours/s", "value": tours_all / (ms / 1e3), "unit": "tours/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "plain AS, n=4096 uniform in [0,100000)^2, m=512, k=32, "
                       "rho=0.1, atomic deposit", "n": 4096, "m": 512, "k": 32,
                       "l2": "tau/eta/choice 3 x 64 MB + dist 64 MB > L2"},
            "stage_ms_per_step": {"construct": stage[1] / args.steps,
                                  "epilogue": stage[2] / args.steps,
                                  "pheromone": stage[4] / args.steps},
            "fallback_rate": fallbacks / max(1, tours * 4095), "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "k_construct_cluster", "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm if hbm else None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if hbm else None,
                         "algorithmic_bytes_per_launch": bytes_c / args.steps,
                         "traffic": profiled_traffic("construct_cluster_as_n4096.md"),
                         "traffic_source": "profiles/construct_cluster_as_n4096.md (ncu)"},
            "best": best, "clocks": clk.summary()}


def _batch_timed(b, iters, chunk):
    """Runs `iters` batch iterations in chunks; returns [(gpu_s, mean best)]."""
    import torch
    trace, total = [], 0.0
    done = 0
    while done < iters:
        step = min(chunk, iters - done)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s.record()
        b.run(step)
        b.synchronize()
        e.record()
        torch.cuda.synchronize()
        total += s.elapsed_time(e) / 1e3
        done += step
        trace.append((total, float(b.glob_best().mean()), done))
    return trace


def run_learned(args, rank, world, local):
    """Learned prior vs plain ACO at equal GPU time (C5)."""
    import torch
    import acogpu_gb300 as aco
    from acogpu_gb300 import _abi, instances
    from acogpu_gb300.prior import EdgePrior
    torch.cuda.set_device(local)
    g = instances.SplitMix64(31)
    train_sizes = (100 + g.integers(args.train_instances, 401)).astype(int)
    p = batch_params()
    t0 = time.perf_counter()
    # Labels: every training instance solved by the plain method for
    # train_iters iterations, in batches of LEARN_CHUNK instances; an edge is
    # positive when it lies on the instance's best tour.
    prior = EdgePrior(seed=17)
    label_gpu_s = 0.0
    for c0 in range(0, len(train_sizes), LEARN_CHUNK):
        train = [instances.uniform_instance(int(n), seed=20_000 + i) if i % 2 == 0 else
                 instances.clustered_instance(int(n), seed=20_000 + i)
                 for i, n in enumerate(train_sizes[c0:c0 + LEARN_CHUNK], start=c0)]
        b = aco.Batch(train, params=p, num_ants=BATCH_CAP)
        b.initialize()
        label_gpu_s += _batch_timed(b, args.train_iters, args.train_iters)[-1][0]
        for i in range(len(train)):
            prior.add_examples(b.colony(i))
        b.close()
    examples, positives = prior.num_examples()
    label_s = time.perf_counter() - t0
    loss0 = prior.train(epochs=1, batch=65536, lr=2e-3, seed=1)
    loss = prior.train(epochs=args.epochs, batch=65536, lr=1e-3, seed=2)
    train_s = time.perf_counter() - t0 - label_s
    # One more epoch on each engine, timed alone; the trained weights are put
    # back afterwards so the evaluation below is unaffected.
    w_trained = prior.weights()
    epoch_s = {}
    for name, eng in (("fused", _abi.ACO_GEMM_FUSED), ("tcgen05_layered", _abi.ACO_GEMM_TCGEN05),
                      ("mma_sync_layered", _abi.ACO_GEMM_MMA_SYNC)):
        prior.set_engine(eng)
        prior.train(epochs=1, batch=65536, lr=1e-6, seed=3)  # warm-up (workspace, maps)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        prior.train(epochs=1, batch=65536, lr=1e-6, seed=3)
        epoch_s[name] = time.perf_counter() - t1
    prior.set_engine(_abi.ACO_GEMM_FUSED)
    prior.set_weights(w_trained)
    # Tensor-core work of one epoch: per edge Z1 (K padded to 16), Z2, dH1,
    # dW2 (N = 128) and dW1 (N = 16), 2 FLOP per multiply-add.
    mlp_flop_per_edge = 2 * 128 * (16 + 128 + 128 + 128 + 16)
    fused_tflops = mlp_flop_per_edge * examples / epoch_s["fused"] / 1e12
    sizes = instances.batch_sizes(args.eval_instances, lo=200, hi=2000, seed=41)
    evals = [instances.uniform_instance(int(n), seed=30_000 + i) if i % 2 == 0 else
             instances.clustered_instance(int(n), seed=30_000 + i) for i, n in enumerate(sizes)]
    plain = aco.Batch(evals, params=p, num_ants=BATCH_CAP)
    plain.initialize()
    plain.autotune()
    plain_trace = _batch_timed(plain, args.plain_iters, 50)
    plain.close()
    t_plain, best_plain = plain_trace[-1][0], plain_trace[-1][1]

    learned = aco.Batch(evals, params=p, num_ants=BATCH_CAP)
    learned.initialize()
    learned.autotune()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for i in range(len(evals)):
        prior.apply(learned.colony(i), floor=0.05)
    e.record()
    torch.cuda.synchronize()
    t_infer = s.elapsed_time(e) / 1e3
    # The learned arm runs until its GPU time (inference included) reaches
    # the plain arm's; the trace also gives its quality at a quarter of the
    # time and when it first matches plain's final quality.
    budget = t_plain - t_infer
    trace, spent, done = [], 0.0, 0
    chunk = 10
    while spent < budget and done < args.plain_iters:
        tr = _batch_timed(learned, chunk, chunk)
        spent += tr[-1][0]
        done += chunk
        trace.append((t_infer + spent, tr[-1][1], done))
    learned.close()
    prior.close()
    within = [v for t, v, _ in trace if t <= t_plain * 1.0001]
    best_learned = within[-1] if within else float("nan")
    reach = next((t for t, v, _ in trace if v <= best_plain * 1.001), None)
    q_learned = [v for t, v, _ in trace if t <= 0.25 * t_plain]
    q_plain = [v for t, v, _ in plain_trace if t <= 0.25 * t_plain]
    gap_quarter = (100.0 * (q_learned[-1] - q_plain[-1]) / q_plain[-1]
                   if q_learned and q_plain else None)
    if rank != 0:
        return None
    return {"metric": "tour-length gap at equal GPU time (learned prior vs plain)",
            "value": 100.0 * (best_learned - best_plain) / best_plain, "unit": "%",
            "higher_is_better": False, "n_gpus": world, "data": "synthetic", "dtype": "bf16+f32",
            "config": {"workload": "learned edge prior: "
                       f"{len(train_sizes)} training instances n in [100,500] labelled by "
                       f"{args.train_iters}-iteration plain best tours; {len(evals)} evaluation "
                       f"instances n log-uniform [200,2000]; plain {args.plain_iters} iterations "
                       "vs learned at the same GPU time (inference included)", "k": BATCH_K,
                       "ants_cap": BATCH_CAP},
            "plain": {"gpu_s": t_plain, "iterations": args.plain_iters, "mean_best": best_plain,
                      "trace": plain_trace[::max(1, len(plain_trace) // 10)]},
            "learned": {"gpu_s": trace[-1][0] if trace else None, "iterations": done,
                        "inference_s": t_infer, "mean_best": best_learned,
                        "gap_pct_at_quarter_time": gap_quarter,
                        "reaches_plain_within_0.1pct_at_s": reach,
                        "trace": trace[::max(1, len(trace) // 10)]},
            "training": {"instances": int(len(train_sizes)),
                         "label_iterations": args.train_iters,
                         "label_gpu_s": label_gpu_s, "label_wall_s": label_s,
                         "examples": examples, "positives": positives, "loss_first_epoch": loss0,
                         "loss_last_epoch": loss, "train_wall_s": train_s,
                         "epoch_s_by_engine": epoch_s,
                         "tensor_flop_per_edge": mlp_flop_per_edge,
                         "fused_epoch_tflops": fused_tflops,
                         "fused_epoch_frac_of_measured_bf16": fused_tflops /
                         peaks().get("bf16_tflops", 1900.0)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default per workload, see DEFAULT_STEPS)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="parity_batch8",
                    choices=("parity_batch8", "rbas_aging_n1000", "batch512", "learned",
                             "large4096"))
    ap.add_argument("--batch-instances", type=int, default=BATCH_COUNT,
                    help="instances of the uneven batch per GPU (batch512)")
    ap.add_argument("--train-instances", type=int, default=20_000)
    ap.add_argument("--train-iters", type=int, default=1000)
    ap.add_argument("--eval-instances", type=int, default=256)
    ap.add_argument("--plain-iters", type=int, default=1000)
    ap.add_argument("--epochs", type=int, default=4)
    args = ap.parse_args()
    if args.steps is None:
        args.steps = DEFAULT_STEPS[args.workload]
    world, rank, local = dist_env()
    if args.impl == "reference":
        if args.workload == "parity_batch8":
            out = run_reference_parity(args, rank)
        elif args.workload == "batch512":
            out = run_reference_batch(args, rank)
        else:
            out = run_reference(args, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    try:
        fn = {"batch512": run_batch, "learned": run_learned, "large4096": run_large,
              "rbas_aging_n1000": run_ours, "parity_batch8": run_parity}[args.workload]
        out = fn(args, rank, world, local)
        if out is not None:
            # the CPU baseline: rank 0 of a one-GPU run only
            if fn is run_ours and not args.no_cpu_baseline and world == 1:
                out["cpu_baseline"] = cpu_baseline()
            if fn is run_parity and not args.no_cpu_baseline and world == 1:
                out["cpu_baseline"] = parity_cpu_baseline()
            if fn is run_batch and not args.no_cpu_baseline and world == 1:
                v, threads, desc = batch_cpu_sample(iters=1, per_stratum=1)
                out["cpu_baseline"] = {"value": v, "unit": "tours/s", "cores": threads,
                                       "kind": "port", "sample": desc}
            print(json.dumps(out), flush=True)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
