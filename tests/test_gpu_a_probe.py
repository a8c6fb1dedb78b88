"""Tensor-core layout self-check: one tcgen05.mma on operand images laid out
the way the kernels lay them out must equal A @ B^T.  Only the descriptors
the kernels themselves use are issued; this test runs before any
fused-kernel test."""
import numpy as np
import pytest

from gpu_util import KERNEL_DESC, bf16_round, run_probe, run_probe_tf32, tf32_trunc

pytestmark = pytest.mark.gpu


def test_umma_layout_matches_kernel_convention():
    """kind::f16 (bf16): A MN-major with the 128-byte swizzle (LBO 2048 B,
    SBO 1024 B), B K-major without swizzle (LBO 128 B, SBO 256 B)."""
    rng = np.random.default_rng(5)
    A = bf16_round(rng.standard_normal((128, 16)))
    Bm = bf16_round(rng.standard_normal((16, 16)))
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    D, err = run_probe(A, Bm, KERNEL_DESC)
    assert err == 0 and float(np.abs(D - ref).max()) < 1e-3


def test_umma_tf32_kmajor_layout():
    """kind::tf32 with both fp32 operands K-major, no swizzle (core matrices
    of 8 rows x 16 B, LBO 128 B along k, SBO 256 B between 8-row groups)."""
    rng = np.random.default_rng(6)
    A = tf32_trunc(rng.standard_normal((128, 8)))
    Bm = tf32_trunc(rng.standard_normal((16, 8)))
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    D, err = run_probe_tf32(A, Bm, (128, 256, 0, 128, 256, 0), a_kmajor=True)
    assert err == 0 and float(np.abs(D - ref).max()) < 1e-3


def test_umma_f8_kmajor_layout():
    """kind::f8f6f4 with e4m3 operands, both K-major without swizzle (core
    matrices 8 rows x 16 B, the two 16-byte k halves 128 B apart, 8-row
    groups 256 B apart): the layout of the fp8 tensor tiles.  Products of
    e4m3 values are exact in fp32, so the MMA equals float64 closely."""
    from gpu_util import e4m3_round, run_probe_f8
    rng = np.random.default_rng(8)
    A, Ab = e4m3_round(rng.standard_normal((128, 32)) * 4)
    Bm, Bb = e4m3_round(rng.standard_normal((16, 32)) * 4)
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    D, err = run_probe_f8(Ab, Bb)
    assert err == 0 and float(np.abs(D - ref).max()) < 1e-3 * max(1.0, float(np.abs(ref).max()))


def test_umma_bf16_kmajor_layout():
    """kind::f16 (bf16) with both operands K-major, no swizzle (core matrices
    of 8 rows x 16 B, LBO 128 B along k, SBO 256 B between 8-row groups): the
    layout of the SDDMM block kernel's gathered rows."""
    from gpu_util import run_probe_bf16_kmajor
    rng = np.random.default_rng(9)
    A = bf16_round(rng.standard_normal((128, 16)))
    Bm = bf16_round(rng.standard_normal((16, 16)))
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    D, err = run_probe_bf16_kmajor(A, Bm)
    assert err == 0 and float(np.abs(D - ref).max()) < 1e-3


def test_umma_bf16_kmajor_swizzled_layout():
    """kind::f16 (bf16) with both operands K-major and the 128-byte swizzle
    (128-byte rows of 64 k, 8-row atoms 1024 B apart): the layout of the
    tensor-tile value-gradient kernel's gathered rows."""
    from gpu_util import run_probe_bf16_kmajor_sw128
    rng = np.random.default_rng(10)
    A = bf16_round(rng.standard_normal((128, 16)))
    Bm = bf16_round(rng.standard_normal((16, 16)))
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    D, err = run_probe_bf16_kmajor_sw128(A, Bm)
    assert err == 0 and float(np.abs(D - ref).max()) < 1e-3
