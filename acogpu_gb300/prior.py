"""The learned heuristic prior (include/acogpu.h, aco_prior_*): an
edge-scoring MLP trained on the GPU by the library's own forward and backward
kernels, applied as a multiplier of a colony's candidate heuristic."""
import ctypes

import numpy as np

from .colony import AcoError, Colony, lib

_vp = ctypes.c_void_p
_f32p = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)

FEATURES = 12
HIDDEN = 128
# packed layout: W1[128][12] b1[128] W2[128][128] b2[128] w3[128] b3
SLICES = {}
_off = 0
for _name, _shape in (("W1", (HIDDEN, FEATURES)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)),
                      ("b2", (HIDDEN,)), ("w3", (HIDDEN,)), ("b3", (1,))):
    _size = int(np.prod(_shape))
    SLICES[_name] = (_off, _shape)
    _off += _size
PARAM_COUNT = _off


def unpack(vec):
    return {k: np.asarray(vec[o:o + int(np.prod(s))]).reshape(s) for k, (o, s) in SLICES.items()}


def pack(params):
    out = np.empty(PARAM_COUNT, dtype=np.float32)
    for k, (o, s) in SLICES.items():
        out[o:o + int(np.prod(s))] = np.asarray(params[k], dtype=np.float32).ravel()
    return out


def _setup(L):
    if getattr(L, "_prior_ready", False):
        return
    L.aco_prior_create.argtypes = [ctypes.c_uint64, ctypes.POINTER(_vp)]
    L.aco_prior_param_count.argtypes = []
    for name in ("aco_prior_get_weights", "aco_prior_set_weights"):
        getattr(L, name).argtypes = [_vp, _f32p]
    for name in ("aco_prior_add_examples",):
        getattr(L, name).argtypes = [_vp, _vp]
    L.aco_prior_num_examples.argtypes = [_vp, _i64p, _i64p]
    L.aco_prior_clear_examples.argtypes = [_vp]
    L.aco_prior_train.argtypes = [_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                  ctypes.c_uint64, _f32p]
    L.aco_prior_loss_and_grads.argtypes = [_vp, _f32p, _f32p, ctypes.c_int32, ctypes.c_float,
                                           _f32p, _f32p]
    L.aco_prior_predict.argtypes = [_vp, _f32p, ctypes.c_int32, _f32p]
    L.aco_prior_apply.argtypes = [_vp, _vp, ctypes.c_float]
    L.aco_prior_last_error.argtypes = [_vp]
    L.aco_prior_last_error.restype = ctypes.c_char_p
    L.aco_prior_destroy.argtypes = [_vp]
    L.aco_prior_destroy.restype = None
    L.aco_prior_set_engine.argtypes = [_vp, ctypes.c_int32]
    L.aco_colony_edge_features.argtypes = [_vp, _f32p]
    L.aco_colony_read_candidate_heuristic.argtypes = [_vp, _f32p]
    L._prior_ready = True


def edge_features(colony: Colony):
    """n*k x 12 features of the colony's candidate edges (row i*k + r)."""
    L = lib()
    _setup(L)
    out = np.empty((colony.n * colony.k, FEATURES), dtype=np.float32)
    st = L.aco_colony_edge_features(colony._h, out.ctypes.data_as(_f32p))
    if st:
        raise AcoError(st, "edge_features")
    return out


def candidate_heuristic(colony: Colony):
    """The colony's candidate heuristic (n x k), prior included."""
    L = lib()
    _setup(L)
    out = np.empty((colony.n, colony.k), dtype=np.float32)
    st = L.aco_colony_read_candidate_heuristic(colony._h, out.ctypes.data_as(_f32p))
    if st:
        raise AcoError(st, "candidate_heuristic")
    return out


class EdgePrior:
    """engine: ACO_GEMM_FUSED (default: the whole forward/backward pass of
    each 128-edge tile in one tcgen05 kernel), or the layer-by-layer
    ACO_GEMM_TCGEN05 (TMA + TMEM tensor cores) and ACO_GEMM_MMA_SYNC
    (warp-level mma.sync) GEMM engines."""

    def __init__(self, seed=0, engine=None):
        self._L = lib()
        _setup(self._L)
        self._h = None
        h = _vp()
        st = self._L.aco_prior_create(ctypes.c_uint64(seed), ctypes.byref(h))
        if st:
            raise AcoError(st, "aco_prior_create")
        self._h = h
        if engine is not None:
            self.set_engine(engine)

    def set_engine(self, engine):
        self._check(self._L.aco_prior_set_engine(self._h, int(engine)), "set_engine")

    def _check(self, st, what):
        if st:
            raise AcoError(st, f"{what}: {self._L.aco_prior_last_error(self._h).decode()}")

    def weights(self):
        out = np.empty(PARAM_COUNT, dtype=np.float32)
        self._check(self._L.aco_prior_get_weights(self._h, out.ctypes.data_as(_f32p)), "weights")
        return out

    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == PARAM_COUNT
        self._check(self._L.aco_prior_set_weights(self._h, w.ctypes.data_as(_f32p)), "set")

    def add_examples(self, colony):
        self._check(self._L.aco_prior_add_examples(self._h, colony._h), "add_examples")

    def num_examples(self):
        e, p = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._L.aco_prior_num_examples(self._h, ctypes.byref(e), ctypes.byref(p)),
                    "num_examples")
        return e.value, p.value

    def clear_examples(self):
        self._check(self._L.aco_prior_clear_examples(self._h), "clear")

    def train(self, epochs=3, batch=16384, lr=1e-3, seed=0):
        loss = ctypes.c_float()
        self._check(self._L.aco_prior_train(self._h, int(epochs), int(batch), float(lr),
                                            ctypes.c_uint64(seed), ctypes.byref(loss)), "train")
        return loss.value

    def loss_and_grads(self, feats, labels, pos_weight=1.0):
        feats = np.ascontiguousarray(feats, dtype=np.float32)
        labels = np.ascontiguousarray(labels, dtype=np.float32)
        loss = ctypes.c_float()
        g = np.empty(PARAM_COUNT, dtype=np.float32)
        self._check(self._L.aco_prior_loss_and_grads(
            self._h, feats.ctypes.data_as(_f32p), labels.ctypes.data_as(_f32p), len(labels),
            float(pos_weight), ctypes.byref(loss), g.ctypes.data_as(_f32p)), "loss_and_grads")
        return loss.value, g

    def predict(self, feats):
        feats = np.ascontiguousarray(feats, dtype=np.float32)
        out = np.empty(len(feats), dtype=np.float32)
        self._check(self._L.aco_prior_predict(self._h, feats.ctypes.data_as(_f32p), len(feats),
                                              out.ctypes.data_as(_f32p)), "predict")
        return out

    def apply(self, colony, floor=0.05):
        self._check(self._L.aco_prior_apply(self._h, colony._h, float(floor)), "apply")

    def close(self):
        if self._h:
            self._L.aco_prior_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
