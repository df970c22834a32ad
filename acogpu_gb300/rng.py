"""numpy restatement of the injected uniform stream of include/acogpu_rng.h
(for inspection and tests; the kernels and the oracle use the header)."""
import numpy as np

_U32 = np.uint32


def hash32(x):
    """lowbias32 (Wellons 2018) on uint32 arrays."""
    x = np.asarray(x, dtype=np.uint32)
    with np.errstate(over="ignore"):
        x = x ^ (x >> _U32(16))
        x = x * _U32(0x7FEB352D)
        x = x ^ (x >> _U32(15))
        x = x * _U32(0x846CA68B)
        x = x ^ (x >> _U32(16))
    return x


def ant_key(seed, iteration, ant):
    lo = _U32(seed & 0xFFFFFFFF)
    hi = _U32((seed >> 32) & 0xFFFFFFFF)
    with np.errstate(over="ignore"):
        h = hash32(lo ^ hash32(hi + _U32(0x9E3779B9)))
        h = hash32(h ^ (_U32(iteration & 0xFFFFFFFF) * _U32(0x9E3779B9) + _U32(0x632BE5AB)))
        a = np.asarray(ant, dtype=np.uint32)
        return hash32(h ^ (a * _U32(0x85EBCA6B) + _U32(0xC2B2AE35)))


def uniform_key(key, step):
    with np.errstate(over="ignore"):
        top = hash32(np.asarray(key, dtype=np.uint32) +
                     np.asarray(step, dtype=np.uint32) * _U32(0x9E3779B9)) >> _U32(8)
    u = top.astype(np.float32) * np.float32(2.0 ** -24)
    return np.where(top == 0, np.float32(2.0 ** -25), u)


def uniform(seed, iteration, ant, step):
    return uniform_key(ant_key(seed, iteration, ant), step)


def uniform_grid(seed, iteration, ants, steps):
    k = ant_key(seed, iteration, np.asarray(ants))[:, None]
    return uniform_key(k, np.asarray(steps)[None, :])
