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


def header_enums():
    src = open(os.path.join(ROOT, "include", "acogpu.h")).read()
    return {k: int(v) for k, v in re.findall(r"\b(ACO_[A-Z0-9_]+)\s*=\s*(-?\d+)", src)}


def test_enum_constants_match_the_python_mirror():
    consts = header_enums()
    assert len(consts) >= 40
    mirrored = {k: v for k, v in consts.items() if hasattr(_abi, k)}
    wrong = {k: (v, getattr(_abi, k)) for k, v in mirrored.items() if getattr(_abi, k) != v}
    assert not wrong, wrong
    for k in ("ACO_CONSTRUCT_DIRECT", "ACO_CONSTRUCT_CLUSTER", "ACO_CONSTRUCT_ROWS",
              "ACO_FALLBACK_TIER_AUTO",
              "ACO_FALLBACK_TIER_ON", "ACO_FALLBACK_TIER_OFF", "ACO_ERR_DEVICE_TIMEOUT"):
        assert k in mirrored, k


def test_params_field_order_matches_the_header():
    src = open(os.path.join(ROOT, "include", "acogpu.h")).read()
    body = src[src.index("typedef struct aco_params {"):src.index("} aco_params;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = re.findall(r"^\s*(?:int32_t|uint64_t|float)\s+(\w+)", body, flags=re.M)
    assert names == [f for f, _ in _abi.AcoParams._fields_], names


def test_mode_values_are_checked_before_any_device_call():
    L = aco.lib()
    h = ctypes.c_void_p()
    d = np.zeros((40, 40), np.int32)
    ptr = d.ctypes.data_as(ctypes.c_void_p)
    for field, bad in (("construct_mode", 6), ("construct_mode", -1), ("fallback_tier", 3)):
        p = _abi.default_params(cand_k=20, fallback=_abi.ACO_FALLBACK_BEST)
        setattr(p, field, bad)
        assert L.aco_colony_create(ctypes.byref(p), ptr, 40, 0, ctypes.byref(h)) == \
            _abi.ACO_ERR_INVALID_ARGUMENT, (field, bad)
    # the k <= 32 kernels, forced with a longer candidate list or the full row
    for mode in (_abi.ACO_CONSTRUCT_STAGED, _abi.ACO_CONSTRUCT_DIRECT, _abi.ACO_CONSTRUCT_CLUSTER):
        p = _abi.default_params(cand_k=0, construct_mode=mode)
        assert L.aco_colony_create(ctypes.byref(p), ptr, 40, 0, ctypes.byref(h)) == \
            _abi.ACO_ERR_UNSUPPORTED, mode
    # the long-row kernel: candidate lists longer than 32, n <= 8192
    p = _abi.default_params(cand_k=20, fallback=_abi.ACO_FALLBACK_BEST,
                            construct_mode=_abi.ACO_CONSTRUCT_ROWS)
    assert L.aco_colony_create(ctypes.byref(p), ptr, 40, 0, ctypes.byref(h)) == \
        _abi.ACO_ERR_UNSUPPORTED
    p = _abi.default_params(cand_k=0, construct_mode=_abi.ACO_CONSTRUCT_ROWS)
    big = np.zeros((1, 1), np.int32)
    assert L.aco_colony_create(ctypes.byref(p), big.ctypes.data_as(ctypes.c_void_p), 8193, 0,
                               ctypes.byref(h)) == _abi.ACO_ERR_UNSUPPORTED


def test_null_handles_are_rejected_without_a_device_call():
    """The tuners and the prior's engine switch check their handles first."""
    L = aco.lib()
    t = _abi.AcoTuning()
    L.aco_colony_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(_abi.AcoTuning)]
    L.aco_batch_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(_abi.AcoTuning)]
    L.aco_prior_set_engine.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    assert L.aco_colony_autotune(None, ctypes.byref(t)) == _abi.ACO_ERR_INVALID_ARGUMENT
    assert L.aco_batch_autotune(None, ctypes.byref(t)) == _abi.ACO_ERR_INVALID_ARGUMENT
    for eng in (_abi.ACO_GEMM_MMA_SYNC, _abi.ACO_GEMM_TCGEN05, _abi.ACO_GEMM_FUSED):
        assert L.aco_prior_set_engine(None, eng) == _abi.ACO_ERR_INVALID_ARGUMENT


def test_tuning_layout_matches_c():
    """aco_tuning: five int/float fields, the construction mode, two reserved."""
    assert ctypes.sizeof(_abi.AcoTuning) == 32
    assert _abi.AcoTuning.construct_mode.offset == 20
