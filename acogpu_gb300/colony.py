"""Python mirror of the reference's Colony / AntSystem / RankBasedAntSystem
surface (reference: inc/Colony.h:24-155, inc/AntSystem.h:7-23,
inc/RankBasedAntSystem.h:12-28), bound to the C ABI of include/acogpu.h.

There is no CPU path: if the CUDA library cannot be loaded, constructing a
colony raises.  Errors that the reference turns into exit(EXIT_FAILURE)
(inc/helper_cuda.h:316-325) raise AcoError here.
"""
import ctypes
import os

import numpy as np

from . import _abi
from ._abi import AcoParams, default_params

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libacogpu.so")

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f32p = ctypes.POINTER(ctypes.c_float)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p


class AcoError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


_lib_handle = None


def lib():
    """The loaded engine library (built on first use when nvcc is present)."""
    global _lib_handle
    if _lib_handle is not None:
        return _lib_handle
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"GB300 engine library missing: {LIB_PATH}")
    L = ctypes.CDLL(LIB_PATH)
    L.aco_params_default.argtypes = [ctypes.POINTER(AcoParams)]
    L.aco_params_default.restype = None
    L.aco_colony_create.argtypes = [ctypes.POINTER(AcoParams), _vp, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.POINTER(_vp)]
    L.aco_colony_create_coords.argtypes = [ctypes.POINTER(AcoParams), _f32p, _f32p, ctypes.c_int32,
                                           ctypes.POINTER(_vp)]
    for name in ("aco_colony_initialize", "aco_colony_synchronize"):
        getattr(L, name).argtypes = [_vp]
    L.aco_colony_construct_solution.argtypes = [_vp, _f32p]
    L.aco_colony_run.argtypes = [_vp, ctypes.c_int32]
    for name in ("aco_colony_get_iter_best", "aco_colony_get_glob_best",
                 "aco_colony_get_launch_count"):
        getattr(L, name).argtypes = [_vp, _i64p]
    for name in ("aco_colony_get_num_valid_ants", "aco_colony_get_iteration",
                 "aco_colony_get_reps", "aco_colony_get_best_tour", "aco_colony_read_nn_list",
                 "aco_colony_read_distances", "aco_colony_read_tours"):
        getattr(L, name).argtypes = [_vp, _i32p]
    L.aco_colony_get_size.argtypes = [_vp, _i32p, _i32p, _i32p]
    L.aco_colony_get_params.argtypes = [_vp, ctypes.POINTER(AcoParams)]
    for name in ("aco_colony_set_alpha", "aco_colony_set_beta", "aco_colony_set_rho"):
        getattr(L, name).argtypes = [_vp, ctypes.c_float]
    L.aco_colony_set_optimum.argtypes = [_vp, ctypes.c_int64]
    L.aco_colony_set_rank_w.argtypes = [_vp, ctypes.c_int32]
    L.aco_colony_set_aging_params.argtypes = [_vp, _i32p]
    L.aco_colony_name.argtypes = [_vp]
    L.aco_colony_name.restype = ctypes.c_char_p
    for name in ("aco_colony_read_pheromone", "aco_colony_read_heuristic",
                 "aco_colony_read_choice_info", "aco_colony_write_pheromone"):
        getattr(L, name).argtypes = [_vp, _f32p]
    L.aco_colony_read_tour_lengths.argtypes = [_vp, _i64p]
    L.aco_colony_read_aging.argtypes = [_vp, _i32p, _i32p, _u8p, _f32p, _i32p]
    L.aco_colony_set_stream.argtypes = [_vp, _vp]
    L.aco_colony_get_stats.argtypes = [_vp, ctypes.POINTER(_abi.AcoStats)]
    L.aco_colony_last_error.argtypes = [_vp]
    L.aco_selftest_bounded_wait.argtypes = [ctypes.c_uint32]
    L.aco_debug_fail_allocation.argtypes = [ctypes.c_int32]
    L.aco_debug_fail_allocation.restype = None
    L.aco_colony_last_error.restype = ctypes.c_char_p
    L.aco_status_string.argtypes = [ctypes.c_int]
    L.aco_status_string.restype = ctypes.c_char_p
    L.aco_colony_destroy.argtypes = [_vp]
    L.aco_colony_destroy.restype = None
    L.aco_batch_create.argtypes = [ctypes.POINTER(AcoParams), ctypes.c_int32, _i32p, _f32p,
                                   ctypes.POINTER(_vp)]
    for name in ("aco_batch_initialize", "aco_batch_synchronize"):
        getattr(L, name).argtypes = [_vp]
    L.aco_batch_run.argtypes = [_vp, ctypes.c_int32]
    L.aco_batch_autotune.argtypes = [_vp, ctypes.POINTER(_abi.AcoTuning)]
    L.aco_colony_autotune.argtypes = [_vp, ctypes.POINTER(_abi.AcoTuning)]
    L.aco_batch_set_tuning.argtypes = [_vp, ctypes.c_int32, ctypes.c_int32]
    L.aco_batch_get_size.argtypes = [_vp, _i32p]
    L.aco_batch_get_colony.argtypes = [_vp, ctypes.c_int32, ctypes.POINTER(_vp)]
    for name in ("aco_batch_get_glob_best", "aco_batch_get_tours_built",
                 "aco_batch_get_launch_count"):
        getattr(L, name).argtypes = [_vp, _i64p]
    L.aco_batch_last_error.argtypes = [_vp]
    L.aco_batch_last_error.restype = ctypes.c_char_p
    L.aco_batch_destroy.argtypes = [_vp]
    L.aco_batch_destroy.restype = None
    _lib_handle = L
    return L


def _p(a, t):
    return a.ctypes.data_as(t)


class Colony:
    """One ACO colony on the current GPU (Colony, inc/Colony.h:24-155).

    ``distances`` is an n x n int32 EUC_2D matrix with 0x7fffffff on the
    diagonal (numpy array, or a device pointer as int with
    ``distances_on_device=True``); alternatively pass ``coords=(x, y)`` and
    the matrix is built on the GPU.
    """

    def __init__(self, distances=None, num_cities=None, num_ants=10, params=None, coords=None,
                 distances_on_device=False, **overrides):
        L = lib()
        self._L = L
        self._h = None
        p = params if params is not None else default_params()
        p = AcoParams.from_buffer_copy(p)
        p.num_ants = int(num_ants)
        for k, v in overrides.items():
            setattr(p, k, v)
        h = _vp()
        if coords is not None:
            x = np.ascontiguousarray(coords[0], dtype=np.float32)
            y = np.ascontiguousarray(coords[1], dtype=np.float32)
            n = len(x)
            st = L.aco_colony_create_coords(ctypes.byref(p), _p(x, _f32p), _p(y, _f32p), n,
                                            ctypes.byref(h))
        elif distances_on_device:
            n = int(num_cities)
            st = L.aco_colony_create(ctypes.byref(p), _vp(int(distances)), n, 1, ctypes.byref(h))
        else:
            d = np.ascontiguousarray(distances, dtype=np.int32)
            n = d.shape[0] if num_cities is None else int(num_cities)
            if d.size != n * n:
                raise ValueError("distances must be an n x n matrix")
            st = L.aco_colony_create(ctypes.byref(p), _p(d, _vp), n, 0, ctypes.byref(h))
        if st != 0:
            raise AcoError(st, "aco_colony_create: " + L.aco_status_string(st).decode())
        self._h = h
        self.n = n
        self.m = p.num_ants
        nn_k = ctypes.c_int32()
        L.aco_colony_get_size(h, None, None, ctypes.byref(nn_k))
        self.k = nn_k.value
        self.params = p

    # -- error handling
    def _check(self, st, what):
        if st != 0:
            msg = self._L.aco_colony_last_error(self._h).decode() if self._h else ""
            raise AcoError(st, f"{what}: {msg or self._L.aco_status_string(st).decode()}")

    # -- reference surface (inc/Colony.h:31-49,152)
    def initialize(self):
        self._check(self._L.aco_colony_initialize(self._h), "initialize")

    def constructSolution(self, timers=None):
        """One iteration.  With ``timers`` (a list, or True) the six stage
        times in ms are returned, indexed like the reference's StatsTimer."""
        if timers is None:
            self._check(self._L.aco_colony_construct_solution(self._h, None), "constructSolution")
            return None
        t = np.zeros(6, dtype=np.float32)
        self._check(self._L.aco_colony_construct_solution(self._h, _p(t, _f32p)),
                    "constructSolution")
        if isinstance(timers, list):
            timers[:] = t.tolist()
        return t

    def run(self, iterations):
        """`iterations` graph-replayed iterations, asynchronous."""
        self._check(self._L.aco_colony_run(self._h, int(iterations)), "run")

    def synchronize(self):
        self._check(self._L.aco_colony_synchronize(self._h), "synchronize")

    def autotune(self):
        """Times the construction kernels and launch shapes that build the
        same tours, keeps the fastest and resets the colony to its
        initialised state (aco_colony_autotune)."""
        t = _abi.AcoTuning()
        self._check(self._L.aco_colony_autotune(self._h, ctypes.byref(t)), "autotune")
        return {"ants_per_block": t.ants_per_block, "construct_ms": t.construct_ms,
                "construct_mode": t.construct_mode, "staged": bool(t.staged_instances)}

    def _i64(self, fn):
        v = ctypes.c_int64()
        self._check(fn(self._h, ctypes.byref(v)), fn.__name__)
        return v.value

    def _i32(self, fn):
        v = ctypes.c_int32()
        self._check(fn(self._h, ctypes.byref(v)), fn.__name__)
        return v.value

    def getIterBestDist(self):
        return self._i64(self._L.aco_colony_get_iter_best)

    def getGlobBestDist(self):
        return self._i64(self._L.aco_colony_get_glob_best)

    def getNumValidAnts(self):
        return self._i32(self._L.aco_colony_get_num_valid_ants)

    def getReps(self):
        return self._i32(self._L.aco_colony_get_reps)

    def getIteration(self):
        return self._i32(self._L.aco_colony_get_iteration)

    def stats(self):
        s = _abi.AcoStats()
        self._check(self._L.aco_colony_get_stats(self._h, ctypes.byref(s)), "stats")
        return {f: getattr(s, f) for f, _ in _abi.AcoStats._fields_ if f != "reserved"}

    def set_stream(self, stream_handle):
        """Run on an existing CUDA stream (cudaStream_t as int)."""
        self._check(self._L.aco_colony_set_stream(self._h, _vp(int(stream_handle))), "set_stream")

    def launch_count(self):
        return self._i64(self._L.aco_colony_get_launch_count)

    def getNumAnts(self):
        return self.m

    def getNumCities(self):
        return self.n

    def _params(self):
        p = AcoParams()
        self._check(self._L.aco_colony_get_params(self._h, ctypes.byref(p)), "get_params")
        return p

    def getAlpha(self):
        return self._params().alpha

    def getBeta(self):
        return self._params().beta

    def getRho(self):
        return self._params().rho

    def setAlpha(self, v):
        self._check(self._L.aco_colony_set_alpha(self._h, float(v)), "setAlpha")

    def setBeta(self, v):
        self._check(self._L.aco_colony_set_beta(self._h, float(v)), "setBeta")

    def setRho(self, v):
        self._check(self._L.aco_colony_set_rho(self._h, float(v)), "setRho")

    def setOptimum(self, v):
        self._check(self._L.aco_colony_set_optimum(self._h, int(v)), "setOptimum")

    def antSystemName(self):
        return self._L.aco_colony_name(self._h).decode()

    def getTour(self):
        """Best-so-far tour as the reference prints it: 1-based, comma after
        each city (src/Colony.cu:1173-1180)."""
        return "".join(f"{c + 1}," for c in self.best_tour())

    # -- checkpoint / resume
    def save(self, path):
        """Writes the state the next iterations depend on (aco_colony_save)."""
        self._L.aco_colony_save.argtypes = [_vp, ctypes.c_char_p]
        self._check(self._L.aco_colony_save(self._h, str(path).encode()), "save")

    def load(self, path):
        """Restores a checkpoint of the same instance and parameters into this
        initialized colony; it then continues bit for bit (aco_colony_load)."""
        self._L.aco_colony_load.argtypes = [_vp, ctypes.c_char_p]
        self._check(self._L.aco_colony_load(self._h, str(path).encode()), "load")

    # -- aging surface (inc/Colony.h:128-139)
    def set_aging_params(self, six):
        a = np.ascontiguousarray(six, dtype=np.int32)
        self._check(self._L.aco_colony_set_aging_params(self._h, _p(a, _i32p)), "set_aging")

    # -- state export
    def _mat_f32(self, fn, cols=None):
        out = np.empty((self.n, cols or self.n), dtype=np.float32)
        self._check(fn(self._h, _p(out, _f32p)), fn.__name__)
        return out

    def pheromone(self):
        return self._mat_f32(self._L.aco_colony_read_pheromone)

    def set_pheromone(self, tau):
        tau = np.ascontiguousarray(tau, dtype=np.float32)
        self._check(self._L.aco_colony_write_pheromone(self._h, _p(tau, _f32p)), "write_pheromone")

    def heuristic(self):
        return self._mat_f32(self._L.aco_colony_read_heuristic)

    def choice_info(self):
        return self._mat_f32(self._L.aco_colony_read_choice_info)

    def nn_list(self):
        out = np.empty((self.n, self.k), dtype=np.int32)
        self._check(self._L.aco_colony_read_nn_list(self._h, _p(out, _i32p)), "nn_list")
        return out

    def distances(self):
        out = np.empty((self.n, self.n), dtype=np.int32)
        self._check(self._L.aco_colony_read_distances(self._h, _p(out, _i32p)), "distances")
        return out

    def tours(self):
        out = np.empty((self.m, self.n), dtype=np.int32)
        self._check(self._L.aco_colony_read_tours(self._h, _p(out, _i32p)), "tours")
        return out

    def tour_lengths(self):
        out = np.empty(self.m, dtype=np.int64)
        self._check(self._L.aco_colony_read_tour_lengths(self._h, _p(out, _i64p)), "lengths")
        return out

    def best_tour(self):
        out = np.empty(self.n, dtype=np.int32)
        self._check(self._L.aco_colony_get_best_tour(self._h, _p(out, _i32p)), "best_tour")
        return out

    def aging_state(self):
        age = np.empty(self.m, np.int32)
        perf = np.empty(self.m, np.int32)
        valid = np.empty(self.m, np.uint8)
        mean = np.empty(self.n, np.float32)
        misc = np.empty(2, np.int32)
        self._check(self._L.aco_colony_read_aging(self._h, _p(age, _i32p), _p(perf, _i32p),
                                                  _p(valid, _u8p), _p(mean, _f32p),
                                                  _p(misc, _i32p)), "aging")
        return dict(age=age, perf=perf, valid=valid, mean=mean, isconverged=int(misc[0]),
                    globalperformance=int(misc[1]))

    def close(self):
        if self._h:
            self._L.aco_colony_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AntSystem(Colony):
    """AntSystem(distances, numCities, numAnts, alpha, beta, rho[, minRetirementAge,
    maxRetirementAge, localPeformance, globalPerformance, minPopulationLimit,
    maxPopulationLimit]) -- src/AntSystem.cu:160-182.  Passing the six aging
    values selects the aging variant."""

    def __init__(self, distances, num_cities, num_ants, alpha=1.0, beta=5.0, rho=0.1, *aging,
                 params=None, **options):
        p = params if params is not None else default_params()
        p = AcoParams.from_buffer_copy(p)
        p.variant = _abi.ACO_ANT_SYSTEM
        p.alpha, p.beta, p.rho = alpha, beta, rho
        if aging:
            if len(aging) != 6:
                raise TypeError("the aging constructor takes six aging parameters")
            p.aging = 1
            (p.min_retirement_age, p.max_retirement_age, p.local_performance,
             p.global_performance, p.min_population_limit, p.max_population_limit) = aging
        super().__init__(distances, num_cities, num_ants, params=p, **options)


class RankBasedAntSystem(Colony):
    """RankBasedAntSystem(distances, cities, ants) with setW/getW
    (src/RankBasedAntSystem.cu:14-67); the update follows the published
    rank-based Ant System because the reference's is an empty stub."""

    def __init__(self, distances, cities, ants, params=None, **options):
        p = params if params is not None else default_params()
        p = AcoParams.from_buffer_copy(p)
        p.variant = _abi.ACO_RANK_BASED
        super().__init__(distances, cities, ants, params=p, **options)

    def setW(self, w):
        self._check(self._L.aco_colony_set_rank_w(self._h, int(w)), "setW")

    def getW(self):
        return self._params().rank_w


class _BorrowedColony(Colony):
    """Read-only view of one instance of a Batch (no ownership)."""

    def __init__(self, L, handle, params):
        self._L = L
        self._h = handle
        n, m, k = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        L.aco_colony_get_size(handle, ctypes.byref(n), ctypes.byref(m), ctypes.byref(k))
        self.n, self.m, self.k = n.value, m.value, k.value
        self.params = params

    def close(self):
        self._h = None  # owned by the batch


class Batch:
    """Many instances advanced together (include/acogpu.h, aco_batch_*).

    ``instances`` is a list of (x, y) coordinate arrays; instance i gets
    min(num_ants, n_i) ants and seed params.seed + i * 0x9E3779B97F4A7C15.
    """

    def __init__(self, instances, params=None, num_ants=1024, **overrides):
        L = lib()
        self._L = L
        self._h = None
        p = params if params is not None else default_params()
        p = AcoParams.from_buffer_copy(p)
        p.num_ants = int(num_ants)
        for k, v in overrides.items():
            setattr(p, k, v)
        sizes = np.array([len(x) for x, _ in instances], dtype=np.int32)
        coords = np.concatenate([np.concatenate([np.asarray(x, np.float32),
                                                 np.asarray(y, np.float32)])
                                 for x, y in instances]).astype(np.float32)
        h = _vp()
        st = L.aco_batch_create(ctypes.byref(p), len(sizes), _p(sizes, _i32p), _p(coords, _f32p),
                                ctypes.byref(h))
        if st != 0:
            raise AcoError(st, "aco_batch_create: " + L.aco_status_string(st).decode())
        self._h = h
        self.sizes = sizes
        self.params = p

    def _check(self, st, what):
        if st != 0:
            msg = self._L.aco_batch_last_error(self._h).decode() if self._h else ""
            raise AcoError(st, f"{what}: {msg or self._L.aco_status_string(st).decode()}")

    def __len__(self):
        return len(self.sizes)

    def initialize(self):
        self._check(self._L.aco_batch_initialize(self._h), "batch initialize")

    def run(self, iterations):
        self._check(self._L.aco_batch_run(self._h, int(iterations)), "batch run")

    def synchronize(self):
        self._check(self._L.aco_batch_synchronize(self._h), "batch synchronize")

    def autotune(self):
        t = _abi.AcoTuning()
        self._check(self._L.aco_batch_autotune(self._h, ctypes.byref(t)), "batch autotune")
        return {"ants_per_block": t.ants_per_block, "row_threads": t.row_threads,
                "construct_ms": t.construct_ms, "rows_ms": t.rows_ms,
                "staged_instances": t.staged_instances}

    def set_tuning(self, ants_per_block, row_threads=0):
        self._check(self._L.aco_batch_set_tuning(self._h, int(ants_per_block), int(row_threads)),
                    "batch set_tuning")

    def glob_best(self):
        out = np.empty(len(self.sizes), dtype=np.int64)
        self._check(self._L.aco_batch_get_glob_best(self._h, _p(out, _i64p)), "batch glob_best")
        return out

    def tours_built(self):
        v = ctypes.c_int64()
        self._check(self._L.aco_batch_get_tours_built(self._h, ctypes.byref(v)), "tours_built")
        return v.value

    def launch_count(self):
        v = ctypes.c_int64()
        self._check(self._L.aco_batch_get_launch_count(self._h, ctypes.byref(v)), "launches")
        return v.value

    def colony(self, i):
        h = _vp()
        self._check(self._L.aco_batch_get_colony(self._h, int(i), ctypes.byref(h)), "colony")
        return _BorrowedColony(self._L, h, self.params)

    def close(self):
        if self._h:
            self._L.aco_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
