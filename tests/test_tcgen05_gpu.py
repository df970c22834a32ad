"""GPU test of the tcgen05 GEMM of the MLP (TMA-staged BF16 operands, TMEM
accumulator) against numpy and against the warp-level mma.sync kernel."""
import ctypes

import numpy as np
import pytest

import acogpu_gb300 as aco

pytestmark = pytest.mark.gpu
MMA_SYNC, TCGEN05 = 0, 1


def bf16_bits(a):
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def from_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def gemm(A, B, splits, engine):
    L = aco.lib()
    f = L.aco_gemm_bf16_tn
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                  ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    M, K = A.shape
    N = B.shape[0]
    C = np.empty((M, N), np.float32)
    st = f(A.ctypes.data, B.ctypes.data, C.ctypes.data, M, N, K, splits, engine)
    assert st == 0, st
    return C


@pytest.mark.parametrize("M,N,K,splits", [(128, 128, 64, 1), (256, 128, 128, 1),
                                          (1000, 128, 16, 1), (128, 128, 4096, 8),
                                          (128, 16, 4096, 8), (300, 16, 200, 1)])
def test_tcgen05_gemm_matches_numpy_and_mma_sync(M, N, K, splits):
    rng = np.random.default_rng(M + N + K)
    A = bf16_bits(rng.normal(size=(M, K)))
    B = bf16_bits(rng.normal(size=(N, K)))
    ref = from_bits(A).astype(np.float64) @ from_bits(B).astype(np.float64).T
    tc = gemm(A, B, splits, TCGEN05)
    mm = gemm(A, B, splits, MMA_SYNC)
    scale = np.abs(ref).max()
    assert np.max(np.abs(tc - ref)) <= 1e-4 * scale * max(1, K / 64), "tcgen05 vs numpy"
    assert np.max(np.abs(mm - ref)) <= 1e-4 * scale * max(1, K / 64), "mma.sync vs numpy"
