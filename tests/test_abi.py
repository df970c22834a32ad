"""CPU checks of the C ABI: the library builds, loads, and exports every
function include/acogpu.h declares; the ctypes layout matches the C one.
No compute calls (no GPU here)."""
import ctypes
import os
import re

import numpy as np

import acogpu_gb300 as aco
from acogpu_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"^ACO_API\s+[\w\s\*]+?\b(aco_\w+)\s*\(", src, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    L = aco.lib()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_params_default_layout_matches_c():
    L = aco.lib()
    p = _abi.AcoParams()
    L.aco_params_default(ctypes.byref(p))
    assert bytes(p) == bytes(_abi.default_params())
    assert ctypes.sizeof(p) == 128


def test_status_strings_and_invalid_arguments():
    L = aco.lib()
    assert L.aco_status_string(0) == b"ok"
    h = ctypes.c_void_p()
    d = np.zeros((2, 2), np.int32)
    p = _abi.default_params()
    # n < 3 is rejected before any device call
    assert L.aco_colony_create(ctypes.byref(p), d.ctypes.data_as(ctypes.c_void_p), 2, 0,
                               ctypes.byref(h)) == _abi.ACO_ERR_INVALID_ARGUMENT
    p.cand_k, p.fallback = 5, _abi.ACO_FALLBACK_REFERENCE
    d = np.zeros((10, 10), np.int32)
    assert L.aco_colony_create(ctypes.byref(p), d.ctypes.data_as(ctypes.c_void_p), 10, 0,
                               ctypes.byref(h)) == _abi.ACO_ERR_UNSUPPORTED
