"""TEST INFRASTRUCTURE: loaders for the CPU checkers of the GB300 ACO engine.

* ``Port`` -- the C restatement in ``aco_oracle.c`` (built into
  ``oracle/_build``), available wherever gcc is.
* ``Ref`` -- the reference's own CPU AntSystem compiled in place from its
  sources (``oracle/Makefile ref`` into ``oracle/_ref``); available only where
  the reference sources are.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package.  The product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

from acogpu_gb300._abi import AcoParams, aging_six

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libaco_oracle.so")
REF_SO = {False: os.path.join(HERE, "_ref", "libacoref_noaging.so"),
          True: os.path.join(HERE, "_ref", "libacoref_aging.so")}
# The reference checkout: ACO_REFERENCE_DIR, else a `reference` directory
# beside this repository.  Absent on machines without it (the checks that
# need it are skipped there).
REF_SOURCES = (os.environ.get("ACO_REFERENCE_DIR")
               or os.path.normpath(os.path.join(HERE, os.pardir, os.pardir, "reference")))

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f32p = ctypes.POINTER(ctypes.c_float)
_u8p = ctypes.POINTER(ctypes.c_uint8)


def _ptr(a, t):
    return a.ctypes.data_as(t)


def build_port(force=False):
    if force or not os.path.exists(PORT_SO):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def ref_available():
    return os.path.isdir(os.path.join(REF_SOURCES, "src")) or all(
        os.path.exists(p) for p in REF_SO.values())


def build_ref():
    if not all(os.path.exists(p) for p in REF_SO.values()):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SOURCES}", "-j4"],
                       check=True)


_port_lib = None


def port_lib():
    global _port_lib
    if _port_lib is None:
        build_port()
        L = ctypes.CDLL(PORT_SO)
        L.oc_create.argtypes = [ctypes.POINTER(AcoParams), _i32p, ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_void_p)]
        L.oc_iter_best.restype = ctypes.c_int64
        L.oc_glob_best.restype = ctypes.c_int64
        L.oc_fallback_count.restype = ctypes.c_int64
        L.oc_tau0.restype = ctypes.c_float
        L.oc_heuristic.restype = ctypes.c_float
        L.oc_heuristic.argtypes = [ctypes.c_int32, ctypes.c_float, ctypes.c_int32]
        L.oc_greedy_length.restype = ctypes.c_int64
        for f in ("oc_initialize", "oc_iterate", "oc_destroy", "oc_iter_best", "oc_glob_best",
                  "oc_num_valid", "oc_cand_k", "oc_tau0", "oc_fallback_count"):
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.oc_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        _port_lib = L
    return _port_lib


def distances(x, y):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    n = len(x)
    out = np.empty((n, n), dtype=np.int32)
    port_lib().oc_distances(_ptr(x, _f32p), _ptr(y, _f32p), ctypes.c_int32(n), _ptr(out, _i32p))
    return out


def nn_rows(dist, order):
    dist = np.ascontiguousarray(dist, dtype=np.int32)
    n = dist.shape[0]
    out = np.empty((n, n), dtype=np.int32)
    port_lib().oc_nn_rows(_ptr(dist, _i32p), ctypes.c_int32(n), ctypes.c_int32(order),
                          _ptr(out, _i32p))
    return out


def heuristic(d, beta, mode):
    return port_lib().oc_heuristic(int(d), float(beta), int(mode))


def greedy_length(dist):
    dist = np.ascontiguousarray(dist, dtype=np.int32)
    return port_lib().oc_greedy_length(_ptr(dist, _i32p), ctypes.c_int32(dist.shape[0]))


def pheromone_update_f64(tau, rho, tours, lens, weights):
    tau = np.ascontiguousarray(tau, dtype=np.float64)
    tours = np.ascontiguousarray(tours, dtype=np.int32)
    lens = np.ascontiguousarray(lens, dtype=np.int64)
    weights = np.ascontiguousarray(weights, dtype=np.float64)
    n = tau.shape[0]
    port_lib().oc_pheromone_update_f64(
        tau.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_int32(n),
        ctypes.c_double(rho), ctypes.c_int32(len(lens)), _ptr(tours, _i32p),
        _ptr(lens, _i64p), weights.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return tau


class Port:
    """The C restatement, one colony."""

    def __init__(self, params: AcoParams, dist, threads=1):
        self.L = port_lib()
        self.dist = np.ascontiguousarray(dist, dtype=np.int32)
        self.n = self.dist.shape[0]
        self.m = params.num_ants
        self.params = params
        h = ctypes.c_void_p()
        st = self.L.oc_create(ctypes.byref(params), _ptr(self.dist, _i32p), self.n, ctypes.byref(h))
        if st != 0:
            raise ValueError(f"oc_create failed with status {st}")
        self.h = h
        self.k = None
        self.L.oc_set_threads(self.h, threads)

    def initialize(self):
        self.L.oc_initialize(self.h)
        self.k = self.L.oc_cand_k(self.h)

    def iterate(self, count=1):
        for _ in range(count):
            self.L.oc_iterate(self.h)

    def iter_best(self):
        return self.L.oc_iter_best(self.h)

    def glob_best(self):
        return self.L.oc_glob_best(self.h)

    def num_valid(self):
        return self.L.oc_num_valid(self.h)

    def tau0(self):
        return self.L.oc_tau0(self.h)

    def fallbacks(self):
        return self.L.oc_fallback_count(self.h)

    def _nn_f(self, fn):
        out = np.empty((self.n, self.n), dtype=np.float32)
        fn(self.h, _ptr(out, _f32p))
        return out

    def pheromone(self):
        return self._nn_f(self.L.oc_get_pheromone)

    def set_pheromone(self, tau):
        tau = np.ascontiguousarray(tau, dtype=np.float32)
        self.L.oc_set_pheromone(self.h, _ptr(tau, _f32p))

    def heuristic(self):
        return self._nn_f(self.L.oc_get_heuristic)

    def set_candidate_heuristic(self, eta_nk):
        eta_nk = np.ascontiguousarray(eta_nk, dtype=np.float32)
        self.L.oc_set_candidate_heuristic(self.h, _ptr(eta_nk, _f32p))

    def choice(self):
        return self._nn_f(self.L.oc_get_choice)

    def nn(self):
        out = np.empty((self.n, self.k), dtype=np.int32)
        self.L.oc_get_nn(self.h, _ptr(out, _i32p))
        return out

    def tours(self):
        out = np.empty((self.m, self.n), dtype=np.int32)
        self.L.oc_get_tours(self.h, _ptr(out, _i32p))
        return out

    def lengths(self):
        out = np.empty(self.m, dtype=np.int64)
        self.L.oc_get_lengths(self.h, _ptr(out, _i64p))
        return out

    def best_tour(self):
        out = np.empty(self.n, dtype=np.int32)
        self.L.oc_get_best_tour(self.h, _ptr(out, _i32p))
        return out

    def aging(self):
        age = np.empty(self.m, np.int32)
        perf = np.empty(self.m, np.int32)
        valid = np.empty(self.m, np.uint8)
        mean = np.empty(self.n, np.float32)
        misc = np.empty(2, np.int32)
        self.L.oc_get_aging(self.h, _ptr(age, _i32p), _ptr(perf, _i32p), _ptr(valid, _u8p),
                            _ptr(mean, _f32p), _ptr(misc, _i32p))
        return dict(age=age, perf=perf, valid=valid, mean=mean, isconverged=int(misc[0]),
                    globalperformance=int(misc[1]))

    def close(self):
        if self.h:
            self.L.oc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ref_libs = {}


def ref_lib(aging):
    if aging not in _ref_libs:
        build_ref()
        L = ctypes.CDLL(REF_SO[aging])
        L.acoref_create.restype = ctypes.c_void_p
        L.acoref_create.argtypes = [_i32p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, _i32p]
        for f in ("acoref_initialize", "acoref_destroy", "acoref_iter_best", "acoref_glob_best",
                  "acoref_num_valid"):
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.acoref_iterate.argtypes = [ctypes.c_void_p, _f32p]
        L.acoref_set_rng.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.acoref_iter_best.restype = ctypes.c_long
        L.acoref_glob_best.restype = ctypes.c_long
        L.acoref_num_valid.restype = ctypes.c_uint
        L.acoref_draw_count.restype = ctypes.c_long
        _ref_libs[aging] = L
    return _ref_libs[aging]


class Ref:
    """The reference's own CPU AntSystem (noaging or aging build), with the
    injected random stream.  One live instance per build at a time: the
    reference keeps aging state in globals (inc/Colony.cuh:9-12)."""

    def __init__(self, params: AcoParams, dist, stable_nn=False):
        self.aging = bool(params.aging)
        self.L = ref_lib(self.aging)
        self.dist = np.ascontiguousarray(dist, dtype=np.int32)
        self.n = self.dist.shape[0]
        self.m = params.num_ants
        six = np.array(aging_six(params), dtype=np.int32)
        self.L.acoref_set_stable_nn(1 if stable_nn else 0)
        self.h = self.L.acoref_create(_ptr(self.dist, _i32p), self.n, self.m, params.alpha,
                                      params.beta, params.rho, _ptr(six, _i32p))
        self.L.acoref_set_rng(self.h, ctypes.c_uint64(params.seed))

    def initialize(self):
        self.L.acoref_initialize(self.h)

    def iterate(self, count=1):
        t = np.zeros(6, np.float32)
        for _ in range(count):
            self.L.acoref_iterate(self.h, _ptr(t, _f32p))
        return t

    def iter_best(self):
        return self.L.acoref_iter_best(self.h)

    def glob_best(self):
        return self.L.acoref_glob_best(self.h)

    def num_valid(self):
        return self.L.acoref_num_valid(self.h)

    def _nn_f(self, fn):
        out = np.empty((self.n, self.n), dtype=np.float32)
        fn(self.h, _ptr(out, _f32p))
        return out

    def pheromone(self):
        return self._nn_f(self.L.acoref_get_pheromone)

    def heuristic(self):
        return self._nn_f(self.L.acoref_get_heuristic)

    def nn(self):
        out = np.empty((self.n, self.n), dtype=np.int32)
        self.L.acoref_get_nnlist(self.h, _ptr(out, _i32p))
        return out

    def tours(self):
        out = np.empty((self.m, self.n), dtype=np.int32)
        self.L.acoref_get_tours(self.h, _ptr(out, _i32p))
        return out

    def lengths(self):
        out = np.empty(self.m, dtype=np.int64)
        self.L.acoref_get_lengths(self.h, _ptr(out, _i64p))
        return out

    def best_tour(self):
        out = np.empty(self.n, dtype=np.int32)
        self.L.acoref_get_best_tour(self.h, _ptr(out, _i32p))
        return out

    def aging_state(self):
        age = np.empty(self.m, np.int32)
        perf = np.empty(self.m, np.int32)
        valid = np.empty(self.m, np.uint8)
        mean = np.empty(self.n, np.float32)
        misc = np.empty(2, np.int32)
        self.L.acoref_get_aging(self.h, _ptr(age, _i32p), _ptr(perf, _i32p), _ptr(valid, _u8p),
                                _ptr(mean, _f32p), _ptr(misc, _i32p))
        return dict(age=age, perf=perf, valid=valid, mean=mean, isconverged=int(misc[0]),
                    globalperformance=int(misc[1]))

    def close(self):
        if self.h:
            self.L.acoref_destroy(self.h)
            self.h = None
        # The reference prints diagnostics through C stdio ("probability
        # issue" when its walk runs past a row); flush them now, while the
        # caller's output capture is still in place.
        ctypes.CDLL(None).fflush(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
