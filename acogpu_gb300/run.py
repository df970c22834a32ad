"""The run loop of the reference's TSP class (src/TSP.cpp) on the native
aco_execute (include/acogpu.h): termination by time, iterations,
repetitions or optimum, the per-iteration Statistics and the summary."""
import ctypes

from . import _abi
from .colony import lib

_vp = ctypes.c_void_p
INFINITE = 2**31 - 1  # INFINITE_VALUE of the reference defaults (inc/default.h)


def _setup(L):
    if getattr(L, "_run_ready", False):
        return
    L.aco_execute.argtypes = [_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                              ctypes.c_int32, ctypes.c_float,
                              ctypes.POINTER(_abi.IterationStats), ctypes.c_int32,
                              ctypes.POINTER(_abi.RunSummary)]
    L._run_ready = True


def _as_dict(st):
    return {name: getattr(st, name) for name, _ in st._fields_}


class TSP:
    """TSP(maxTime, maxIter, maxReps, optimum) (src/TSP.cpp:8-14); maxTime is
    compared with the summed stage timers in ms.  The reference's defaults:
    maxTime infinite, maxIter 10, optimum -1 (inc/default.h:12-15)."""

    def __init__(self, max_time=INFINITE, max_iter=10, max_reps=INFINITE, optimum=-1):
        self.max_time, self.max_iter = int(max_time), int(max_iter)
        self.max_reps, self.optimum = int(max_reps), int(optimum)

    def execute(self, colony, calcdisttime=0.0, max_stats=None):
        """TSP::execute (src/TSP.cpp:23-79) without the file output: returns
        (per-iteration statistics, summary) as lists of dicts / a dict."""
        L = lib()
        _setup(L)
        cap = self.max_iter if max_stats is None else int(max_stats)
        cap = max(0, min(cap, 1 << 20))
        stats = (_abi.IterationStats * max(cap, 1))()
        summary = _abi.RunSummary()
        st = L.aco_execute(colony._h, self.max_time, self.max_iter, self.max_reps, self.optimum,
                           float(calcdisttime), stats, cap, ctypes.byref(summary))
        colony._check(st, "execute")
        n = min(summary.numiter, cap)
        return [_as_dict(stats[i]) for i in range(n)], _as_dict(summary)
