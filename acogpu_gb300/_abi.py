"""ctypes mirror of ``include/acogpu.h``: the parameter struct and enums.

Pure layout, no library loading, so the CPU oracle and the tests can share
it without touching the GPU library.
"""
import ctypes

ACO_MAX_DISTANCE = 0x7FFFFFFF

# status codes (enum aco_status)
ACO_OK = 0
ACO_ERR_INVALID_ARGUMENT = 1
ACO_ERR_OUT_OF_MEMORY = 2
ACO_ERR_CUDA = 3
ACO_ERR_NOT_INITIALIZED = 4
ACO_ERR_UNSUPPORTED = 5
ACO_ERR_DEVICE_TIMEOUT = 6
ACO_ERR_DEVICE_CHECK = 7
ACO_ERR_IO = 8
ACO_ERR_FORMAT = 9

ACO_ANT_SYSTEM, ACO_RANK_BASED = 0, 1
ACO_NN_STABLE, ACO_NN_REFERENCE_QSORT = 0, 1
ACO_HEURISTIC_DEVICE, ACO_HEURISTIC_LIBM = 0, 1
ACO_FALLBACK_REFERENCE, ACO_FALLBACK_BEST = 0, 1
ACO_DEPOSIT_DETERMINISTIC, ACO_DEPOSIT_ATOMIC = 0, 1
ACO_TAU0_REFERENCE, ACO_TAU0_DORIGO, ACO_TAU0_VALUE = 0, 1, 2
ACO_CONSTRUCT_AUTO, ACO_CONSTRUCT_GLOBAL, ACO_CONSTRUCT_STAGED = 0, 1, 2
ACO_CONSTRUCT_DIRECT, ACO_CONSTRUCT_CLUSTER = 3, 4
ACO_CONSTRUCT_ROWS = 5
ACO_FALLBACK_TIER_AUTO, ACO_FALLBACK_TIER_ON, ACO_FALLBACK_TIER_OFF = 0, 1, 2
ACO_GEMM_MMA_SYNC, ACO_GEMM_TCGEN05, ACO_GEMM_FUSED = 0, 1, 2

TIMER_NAMES = ("init_tour", "tour", "compute_ant_distance", "evaporate_pheromone",
               "update_pheromone", "compute_probabilities")


class AcoParams(ctypes.Structure):
    _fields_ = [
        ("variant", ctypes.c_int32),
        ("num_ants", ctypes.c_int32),
        ("alpha", ctypes.c_float),
        ("beta", ctypes.c_float),
        ("rho", ctypes.c_float),
        ("use_alpha", ctypes.c_int32),
        ("cand_k", ctypes.c_int32),
        ("nn_order", ctypes.c_int32),
        ("heuristic", ctypes.c_int32),
        ("fallback", ctypes.c_int32),
        ("deposit", ctypes.c_int32),
        ("tau0_mode", ctypes.c_int32),
        ("tau0", ctypes.c_float),
        ("rank_w", ctypes.c_int32),
        ("aging", ctypes.c_int32),
        ("min_retirement_age", ctypes.c_int32),
        ("max_retirement_age", ctypes.c_int32),
        ("local_performance", ctypes.c_int32),
        ("global_performance", ctypes.c_int32),
        ("min_population_limit", ctypes.c_int32),
        ("max_population_limit", ctypes.c_int32),
        ("broker", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("ants_per_block", ctypes.c_int32),
        ("construct_mode", ctypes.c_int32),
        ("fallback_tier", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 5),
    ]


class AcoStats(ctypes.Structure):
    _fields_ = [
        ("iteration", ctypes.c_int64),
        ("tours_built", ctypes.c_int64),
        ("fallbacks", ctypes.c_int64),
        ("greedy_length", ctypes.c_int64),
        ("iter_best", ctypes.c_int64),
        ("glob_best", ctypes.c_int64),
        ("num_valid", ctypes.c_int32),
        ("tau0", ctypes.c_float),
        ("reserved", ctypes.c_int64 * 4),
    ]


class AcoTuning(ctypes.Structure):
    _fields_ = [
        ("ants_per_block", ctypes.c_int32),
        ("row_threads", ctypes.c_int32),
        ("construct_ms", ctypes.c_float),
        ("rows_ms", ctypes.c_float),
        ("staged_instances", ctypes.c_int32),
        ("construct_mode", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 2),
    ]


def default_params(**overrides):
    """Reference defaults (inc/default.h, src/Colony.cu:31-36); keyword
    arguments override fields by name."""
    p = AcoParams()
    p.variant = ACO_ANT_SYSTEM
    p.num_ants = 10
    p.alpha, p.beta, p.rho = 1.0, 5.0, 0.1
    p.use_alpha = 0
    p.cand_k = 0
    p.nn_order = ACO_NN_REFERENCE_QSORT
    p.heuristic = ACO_HEURISTIC_LIBM
    p.fallback = ACO_FALLBACK_REFERENCE
    p.deposit = ACO_DEPOSIT_DETERMINISTIC
    p.tau0_mode = ACO_TAU0_REFERENCE
    p.tau0 = 1e-6
    p.rank_w = 5
    p.aging = 0
    (p.min_retirement_age, p.max_retirement_age, p.local_performance,
     p.global_performance, p.min_population_limit, p.max_population_limit) = (30, 50, 10, 10, 40, 100)
    p.broker = 0
    p.seed = 12345678
    p.ants_per_block = 0
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(f"aco_params has no field {k!r}")
        setattr(p, k, v)
    return p


def aging_six(p):
    return (p.min_retirement_age, p.max_retirement_age, p.local_performance,
            p.global_performance, p.min_population_limit, p.max_population_limit)


class IterationStats(ctypes.Structure):
    """aco_iteration_stats: the reference's Statistics (inc/Statistics.h)."""
    _fields_ = [("ants", ctypes.c_int32), ("iter", ctypes.c_int32),
                ("iterbest", ctypes.c_int64), ("globalbest", ctypes.c_int64)] + [
        (name, ctypes.c_float) for name in (
            "t_inittour", "t_computeprob", "t_tour", "t_antdist", "t_evapphoremone",
            "t_updatephoremone", "t_itertime", "t_globaltime")]


class RunSummary(ctypes.Structure):
    """aco_run_summary: the reference's SummaryStatistics without its strings."""
    _fields_ = [("numcities", ctypes.c_int32), ("numants", ctypes.c_int32),
                ("numiter", ctypes.c_int32)] + [
        (name, ctypes.c_float) for name in (
            "t_inittime", "t_inittour", "t_computeprob", "t_tour", "t_antdist", "t_distcalc",
            "t_updatephoremone", "t_evappheromnes", "t_totaltime", "d_optimal", "d_calulated",
            "d_error", "p_alpha", "p_beta", "p_rho")]
