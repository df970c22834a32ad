"""TEST INFRASTRUCTURE: CPU oracle of the learned prior's MLP.

FP64 restatement of the forward and backward pass of the edge-scoring MLP
(12 features -> 128 -> 128 -> 1, ReLU, weighted logistic loss), rounding to
BF16 at the points where the GPU path stores BF16 (inputs, GEMM weights,
hidden activations, the gradients fed to the GEMMs).  `exact=True` drops the
BF16 rounding, for the finite-difference check of the backward pass itself.
Parameter packing: W1[128][12] b1[128] W2[128][128] b2[128] w3[128] b3.
"""
import numpy as np

F, H = 12, 128


def bf16(a):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)),
                        ("w3", (H,)), ("b3", (1,))):
        size = int(np.prod(shape))
        out[name] = w[o:o + size].reshape(shape)
        o += size
    return out


def pack(d):
    return np.concatenate([d[k].ravel() for k in ("W1", "b1", "W2", "b2", "w3", "b3")])


def forward(w, X, exact=False):
    r = (lambda a: np.asarray(a, np.float64)) if exact else bf16
    p = unpack(w)
    Xb = r(X)
    Z1 = Xb @ r(p["W1"]).T + p["b1"]
    H1 = r(np.maximum(Z1, 0.0))
    Z2 = H1 @ r(p["W2"]).T + p["b2"]
    H2 = r(np.maximum(Z2, 0.0))
    z = H2 @ p["w3"] + p["b3"][0]
    return dict(Xb=Xb, H1=H1, H2=H2, z=z)


def loss_and_grads(w, X, y, pos_weight=1.0, exact=False):
    r = (lambda a: np.asarray(a, np.float64)) if exact else bf16
    p = unpack(w)
    f = forward(w, X, exact)
    z, H1, H2, Xb = f["z"], f["H1"], f["H2"], f["Xb"]
    y = np.asarray(y, np.float64)
    wt = np.where(y > 0.5, pos_weight, 1.0)
    norm = max(1, len(y))
    loss = np.sum(wt * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))) / norm
    dz = wt * (1.0 / (1.0 + np.exp(-z)) - y) / norm
    g = {}
    g["w3"] = H2.T @ dz
    g["b3"] = np.array([dz.sum()])
    dZ2f = np.outer(dz, p["w3"]) * (H2 > 0)
    g["b2"] = dZ2f.sum(axis=0)
    dZ2 = r(dZ2f)
    g["W2"] = dZ2.T @ H1
    dH1 = dZ2 @ r(p["W2"])
    dZ1f = dH1 * (H1 > 0)
    g["b1"] = dZ1f.sum(axis=0)
    dZ1 = r(dZ1f)
    g["W1"] = dZ1.T @ Xb
    return loss, pack(g)


def predict(w, X):
    z = forward(w, X)["z"]
    return 1.0 / (1.0 + np.exp(-z))
