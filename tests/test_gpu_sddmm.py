"""SDDMM kernels (1D + block tiles) on the reference's selected plans."""
import numpy as np
import pytest
import torch

from conftest import golden_files
from golden_plan import plan_from_fixture
import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300.ops import DeviceSddmmPlan

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("F", [32, 64, 41, 128, 256, 200])
@pytest.mark.parametrize("path", golden_files("sddmm"), ids=lambda p: p.split("/")[-1][:-4])
def test_sddmm_matches_fp64(path, F):
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    A = S.fixture_matrix(meta, arr)
    dev = D.build_sddmm_device(plan.tiles, A.shape, A.nnz)
    p = DeviceSddmmPlan(dev)
    rng = np.random.default_rng(F)
    X = rng.standard_normal((A.shape[0], F)).astype(np.float32)
    Y = rng.standard_normal((A.shape[1], F)).astype(np.float32)
    out = p.run(torch.as_tensor(X, device="cuda"), torch.as_tensor(Y, device="cuda")).cpu().numpy()
    assert S.rel_fro(out, S.sddmm_fp64(A, X, Y)) <= 1e-5


@pytest.mark.parametrize("F", [64, 41, 128, 200])
@pytest.mark.parametrize("path", golden_files("sddmm"), ids=lambda p: p.split("/")[-1][:-4])
def test_sddmm_bf16_operands_match_fp64(path, F):
    """X and Y in bf16: the block tiles run one bf16 MMA per 16 features on
    the tensor cores, the 1D tiles convert to fp32; products of bf16 values
    are exact in fp32, so the result is fp32-accurate against float64 of the
    same bf16 values.  The tensor-core kernel's error flag stays clear."""
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    A = S.fixture_matrix(meta, arr)
    dev = D.build_sddmm_device(plan.tiles, A.shape, A.nnz)
    p = DeviceSddmmPlan(dev)
    rng = np.random.default_rng(F + 1)
    X = torch.as_tensor(rng.standard_normal((A.shape[0], F)).astype(np.float32), device="cuda").to(torch.bfloat16)
    Y = torch.as_tensor(rng.standard_normal((A.shape[1], F)).astype(np.float32), device="cuda").to(torch.bfloat16)
    out = p.run(X, Y).cpu().numpy()
    assert p.error_flag() == 0
    assert S.rel_fro(out, S.sddmm_fp64(A, X.float().cpu().numpy(), Y.float().cpu().numpy())) <= 1e-5


def test_sddmm_block_only_plan_runs_on_tensor_cores():
    """A plan whose tiles are all blocks (the reference's TC-only search):
    every output comes from the tensor-core block kernel (fp32 operands, hi +
    lo bf16 products), within 1e-5 of float64."""
    path = [p for p in golden_files("sddmm") if p.endswith("sddmm_mask_1024_tc.npz")][0]
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    A = S.fixture_matrix(meta, arr)
    dev = D.build_sddmm_device(plan.tiles, A.shape, A.nnz)
    assert len(dev.mid_idx) == 0 and len(dev.blk_out) == A.nnz
    p = DeviceSddmmPlan(dev)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((A.shape[0], 64)).astype(np.float32)
    Y = rng.standard_normal((A.shape[1], 64)).astype(np.float32)
    out = p.run(torch.as_tensor(X, device="cuda"), torch.as_tensor(Y, device="cuda")).cpu().numpy()
    assert p.error_flag() == 0
    assert S.rel_fro(out, S.sddmm_fp64(A, X, Y)) <= 1e-5
