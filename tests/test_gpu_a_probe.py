"""Tensor-core layout self-check: one tcgen05.mma on operand images laid out
the way the fused kernel lays them out must equal A @ B^T.  The probe keeps
every possible descriptor interpretation inside its shared memory, so this
test runs before any fused-kernel test."""
import numpy as np
import pytest

from gpu_util import KERNEL_DESC, TF32_DESC, bf16_round, run_probe, run_probe_tf32, tf32_trunc

pytestmark = pytest.mark.gpu


def test_umma_layout_matches_kernel_convention():
    rng = np.random.default_rng(5)
    A = bf16_round(rng.standard_normal((128, 16)))
    Bm = bf16_round(rng.standard_normal((16, 16)))
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    report = {}
    for a_lbo, a_sbo in [(2048, 1024), (1024, 2048)]:
        for b_lbo, b_sbo in [(128, 256), (256, 128)]:
            desc = (a_lbo, a_sbo, 2, b_lbo, b_sbo, 0)
            D, err = run_probe(A, Bm, desc)
            report[desc] = (err, float(np.abs(D - ref).max()))
    print("probe report:", report)
    err, maxdiff = report[KERNEL_DESC]
    assert err == 0 and maxdiff < 1e-3, report


def test_umma_tf32_layout():
    """kind::tf32 with both fp32 operands K-major, no swizzle (core matrices
    of 8 rows x 16 B, LBO 128 B along k, SBO 256 B between 8-row groups)
    equals A @ B^T.  The MN-major (feature-contiguous) A variants are only
    reported: on this part they do not give A @ B^T, which is why no SpMM
    tile feeds fp32 B rows to kind::tf32 in place."""
    rng = np.random.default_rng(6)
    A = tf32_trunc(rng.standard_normal((128, 8)))
    Bm = tf32_trunc(rng.standard_normal((16, 8)))
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    report = {}
    for desc in [TF32_DESC, (1024, 2048, 2, 256, 128, 0), (2048, 1024, 2, 128, 256, 0)]:
        D, err = run_probe_tf32(A, Bm, desc)
        report[("mn", desc)] = (err, float(np.abs(D - ref).max()))
    for desc in [(128, 256, 0, 128, 256, 0), (256, 128, 0, 128, 256, 0)]:
        D, err = run_probe_tf32(A, Bm, desc, a_kmajor=True)
        report[("k", desc)] = (err, float(np.abs(D - ref).max()))
    print("tf32 probe report:", report)
    err, maxdiff = report[("k", (128, 256, 0, 128, 256, 0))]
    assert err == 0 and maxdiff < 1e-3, report
