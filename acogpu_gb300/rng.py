"""numpy restatement of the injected uniform stream of include/acogpu_rng.h
(for inspection and tests; the kernels use the header itself)."""
import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def key(iteration, ant, step):
    it = np.uint64(iteration & 0x3FFFFF)
    a = np.asarray(ant, dtype=np.uint64) & np.uint64(0x1FFFFF)
    s = np.asarray(step, dtype=np.uint64) & np.uint64(0x1FFFFF)
    return (it << np.uint64(42)) | (a << np.uint64(21)) | s


def uniform(seed, iteration, ant, step):
    h = mix64(mix64(np.uint64(seed)) ^ key(iteration, ant, step))
    top = (h >> np.uint64(40)).astype(np.uint32)
    u = top.astype(np.float32) * np.float32(2.0 ** -24)
    return np.where(top == 0, np.float32(2.0 ** -25), u)


def uniform_grid(seed, iteration, ants, steps):
    a = np.asarray(ants)[:, None]
    s = np.asarray(steps)[None, :]
    return uniform(seed, iteration, a, s)
