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


def _Net(nz, nx, batch, seed):
    from projectracer_gb300.learned import UNet

    return UNet(nz, nx, batch, seed)


def _smooth_batch(rng, B, nz, nx):
    z, x = np.meshgrid(np.linspace(0, 1, nz), np.linspace(0, 2, nx), indexing="ij")
    xs = np.zeros((B, 4, nz, nx), dtype=np.float32)
    for b in range(B):
        for c in range(4):
            a, kx, kz = rng.uniform(0.5, 1.5), rng.integers(1, 4), rng.integers(1, 4)
            xs[b, c] = a * np.sin(kx * np.pi * x / 2 + rng.uniform(0, 6)) * np.sin(kz * np.pi * z + rng.uniform(0, 6))
    t = (0.5 * xs[:, 0] - 0.3 * xs[:, 3]).astype(np.float32)
    return xs, t


def test_unet_forward_and_gradients_match_cpu_oracle():
    """GPU U-Net (tcgen05 implicit-GEMM convolutions) against the numpy oracle with the same BF16
    rounding points: output, loss and every parameter gradient."""
    import oracle.unet_ref as ur

    nz, nx, B = 16, 32, 2
    net = _Net(nz, nx, B, 11)
    rng = np.random.default_rng(3)
    x, t = _smooth_batch(rng, B, nz, nx)
    p = net.params().astype(np.float64)
    y_gpu = net.forward(x)
    y_ref, _ = ur.forward(p, x)
    assert np.max(np.abs(y_gpu - y_ref)) <= 1e-2 * np.max(np.abs(y_ref))
    loss_gpu, g_gpu = net.gradients(x, t)
    loss_ref, g_ref = ur.gradients(p, x, t)
    assert abs(loss_gpu - loss_ref) <= 1e-2 * loss_ref
    offs, out_w, out_b, total = ur.layout()
    cos = float(g_gpu @ g_ref / (np.linalg.norm(g_gpu) * np.linalg.norm(g_ref)))
    assert cos > 0.999
    for li, (wo, bo) in enumerate(offs):
        for a, b in ((wo, bo), (bo, bo + ur.SPEC[li][4])):
            err = np.linalg.norm(g_gpu[a:b] - g_ref[a:b]) / max(np.linalg.norm(g_ref[a:b]), 1e-30)
            assert err < 3e-2, (li, a == wo, err)
    net.close()


def test_unet_adam_reduces_loss_and_weights_round_trip(tmp_path):
    nz, nx, B = 32, 64, 4
    net = _Net(nz, nx, B, 7)
    rng = np.random.default_rng(9)
    x, t = _smooth_batch(rng, B, nz, nx)
    first = net.train_step(x, t, 1e-3)
    for _ in range(80):
        last = net.train_step(x, t, 1e-3)
    assert last < 0.3 * first
    path = str(tmp_path / "w.bin")
    net.save(path)
    from projectracer_gb300.learned import UNet

    net2 = UNet.load(path, nz, nx, B)
    assert np.array_equal(net.forward(x), net2.forward(x))
    net2.close()
    net.close()
