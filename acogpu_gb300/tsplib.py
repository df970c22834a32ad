"""TSPLIB instances (include/acogpu.h, aco_tsplib_*): the reader of the
reference's TSPReader (src/TSPReader.cu:25-95) -- TYPE TSP/STSP, EUC_2D,
NODE_COORD_SECTION lines read as "%ld %f %f" -- and a colony built from one."""
import ctypes
from dataclasses import dataclass

import numpy as np

from .colony import AcoError, Colony, lib

_vp = ctypes.c_void_p


def _setup(L):
    if getattr(L, "_tsplib_ready", False):
        return
    L.aco_tsplib_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(_vp)]
    L.aco_tsplib_num_nodes.argtypes = [_vp]
    L.aco_tsplib_num_nodes.restype = ctypes.c_int32
    L.aco_tsplib_name.argtypes = [_vp]
    L.aco_tsplib_name.restype = ctypes.c_char_p
    for name in ("aco_tsplib_xcoords", "aco_tsplib_ycoords"):
        getattr(L, name).argtypes = [_vp]
        getattr(L, name).restype = ctypes.POINTER(ctypes.c_float)
    L.aco_tsplib_last_error.argtypes = []
    L.aco_tsplib_last_error.restype = ctypes.c_char_p
    L.aco_tsplib_destroy.argtypes = [_vp]
    L.aco_tsplib_destroy.restype = None
    L._tsplib_ready = True


@dataclass
class Instance:
    """TSPReader::getName / getNumNodes / getXcoords / getYcoords."""
    name: str
    x: np.ndarray  # float32
    y: np.ndarray  # float32

    @property
    def n(self):
        return len(self.x)


def read(path):
    """Reads a .tsp file; raises AcoError (ACO_ERR_IO, ACO_ERR_FORMAT) like the
    reference's read() returning false."""
    L = lib()
    _setup(L)
    h = _vp()
    st = L.aco_tsplib_read(str(path).encode(), ctypes.byref(h))
    if st:
        raise AcoError(st, f"tsplib read: {L.aco_tsplib_last_error().decode()}")
    try:
        n = L.aco_tsplib_num_nodes(h)
        x = np.ctypeslib.as_array(L.aco_tsplib_xcoords(h), shape=(n,)).copy()
        y = np.ctypeslib.as_array(L.aco_tsplib_ycoords(h), shape=(n,)).copy()
        return Instance(L.aco_tsplib_name(h).decode(), x, y)
    finally:
        L.aco_tsplib_destroy(h)


def colony(path, params=None, num_ants=None):
    """A colony on the instance's EUC_2D distances (src/Setup.cpp:54-70),
    computed on the device from the coordinates."""
    inst = read(path)
    if num_ants is None:
        num_ants = params.num_ants if params is not None else 10
    return Colony(coords=(inst.x, inst.y), params=params, num_ants=num_ants)
