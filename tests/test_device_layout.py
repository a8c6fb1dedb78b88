"""The device layout derived from the reference's plans computes A @ B with
the real values (CPU execution of exactly the arrays the kernel reads), every
output row is written (no NaN left from the uninitialised output), owned rows
have one writer, and the nonzero ids cover every nonzero exactly once."""
import numpy as np
import pytest

from conftest import golden_files
from device_exec import spmm_device_exec
from golden_plan import plan_from_fixture
from gpu_util import random_values
import oracle.semantics as S
from stile_gb300 import device as D


@pytest.mark.parametrize("path", golden_files("spmm"), ids=lambda p: p.split("/")[-1][:-4])
def test_device_layout_executes_to_fp64(path):
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    A = random_values(S.fixture_matrix(meta, arr), seed=11)
    dev = D.build_spmm_device(plan.tiles, A, N=meta["N"])
    B = np.random.default_rng(0).standard_normal((A.shape[1], meta["N"]))
    C = spmm_device_exec(dev, B)
    assert not np.isnan(C).any()
    assert S.rel_fro(C, S.spmm_fp64(A, B)) < 1e-6
    # every nonzero id appears: TC entries + live ELL entries (duplicates only
    # for rows withdrawn into whole-row TC tiles, which the ELL side skips)
    ids = np.concatenate([dev.tc_nnz_id[dev.tc_nnz_id >= 0], dev.ell_nnz_id[dev.ell_nnz_id >= 0]])
    assert np.array_equal(np.unique(ids), np.arange(A.nnz))
    assert len(ids) == A.nnz


@pytest.mark.parametrize("shape", [(768, 512), (200, 300)])
def test_column_block_plan_layout(shape):
    """A searched plan with the tensor-core columns kept in order
    (TC_k_notsorted): every tensor-core k-step reads 16 consecutive columns
    from a multiple of 16 (clamped at the last column when K is not a
    multiple of 16) and the layout executes to the float64 product."""
    from stile_gb300 import synthetic as syn
    from stile_gb300.planner import search_spmm
    A = syn.pruned_weight(*shape, sparsity=0.93, block_frac=0.7, seed=3)
    plan = search_spmm(A, 64, tc_k_notsorted=True)
    dev = D.build_spmm_device(plan.tiles, A, N=64)
    cols = dev.tc_cols.astype(np.int64).reshape(-1, 16)
    assert len(cols) > 0
    assert np.all(cols[:, 0] % 16 == 0)
    assert np.array_equal(cols, np.minimum(cols[:, :1] + np.arange(16), A.shape[1] - 1))
    B = np.random.default_rng(1).standard_normal((A.shape[1], 64))
    C = spmm_device_exec(dev, B)
    assert not np.isnan(C).any()
    assert S.rel_fro(C, S.spmm_fp64(A, B)) < 1e-6


def test_bf16_rounding_matches_torch():
    import torch
    x = np.random.default_rng(0).standard_normal(10000).astype(np.float32) * 100
    x[:4] = [0.0, -0.0, 1e-40, 3.0e38]
    ours = D._to_bf16_bits(x)
    ref = torch.as_tensor(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(ours, ref)


def test_operand_image_layout():
    v = np.arange(256, dtype=np.uint16).reshape(1, 16, 16)  # value = n*16 + k
    img = D.operand_image_16bit(v)[0]
    for n in range(16):
        for k in range(16):
            idx = (n // 8) * 128 + (k // 8) * 64 + (n % 8) * 8 + k % 8
            assert img[idx] == n * 16 + k


