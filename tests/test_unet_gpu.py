"""Tensor-core (tcgen05) BF16 GEMM tile and the U-Net built on it, against numpy references."""
import ctypes

import numpy as np
import pytest

from projectracer_gb300 import engine as eng

pytestmark = pytest.mark.gpu


def to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even FP32 -> BF16, as uint16 bit patterns."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16_to_f32(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (300, 64, 200), (257, 256, 64), (128, 128, 576)])
def test_tc_gemm_matches_fp64_reference(M, N, K):
    L = eng.load_library()
    L.pt_tc_gemm_check.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int]
    rng = np.random.default_rng(M + N + K)
    A = to_bf16_bits(rng.standard_normal((M, K)))
    B = to_bf16_bits(rng.standard_normal((N, K)))
    C = np.zeros((M, N), dtype=np.float32)
    rc = L.pt_tc_gemm_check(A.ctypes.data, B.ctypes.data, C.ctypes.data, M, N, K)
    assert rc == 0, L.pt_last_error()
    ref = bf16_to_f32(A).astype(np.float64) @ bf16_to_f32(B).astype(np.float64).T
    # products of BF16 values are exact in FP32; the FP32 accumulation over K terms bounds the error
    assert np.max(np.abs(C - ref)) <= 1e-6 * K * np.max(np.abs(ref))
