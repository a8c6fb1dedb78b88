"""Fused SpMM / dvals / CSR kernels against the FP64 oracle, on the
reference's own selected plans (golden fixtures) with real matrix values."""
import numpy as np
import pytest
import torch

from conftest import golden_files
from golden_plan import plan_from_fixture
from gpu_util import random_values, umma_layout_ok
import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300 import synthetic as syn
from stile_gb300.ops import CsrMatrix, DeviceSpmmPlan

pytestmark = pytest.mark.gpu

SPMM_FIXTURES = golden_files("spmm")


def _case(path, seed=0):
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    A = random_values(S.fixture_matrix(meta, arr), seed=seed)
    return meta, plan, A


def _needs_tc(plan):
    return any(t.template == "TensorCore_template" for t in plan.tiles)


@pytest.mark.parametrize("mode,tol", [(D.TC_BF16, 1e-2), (D.TC_F16, 2e-3), (D.TC_SPLIT_BF16, 1e-5)],
                         ids=["bf16", "f16", "split"])
@pytest.mark.parametrize("path", SPMM_FIXTURES, ids=lambda p: p.split("/")[-1][:-4])
def test_fused_spmm_matches_fp64(path, mode, tol):
    meta, plan, A = _case(path)
    if _needs_tc(plan) and not umma_layout_ok():
        pytest.fail("tensor-core layout probe failed; fused kernel not run")
    N = meta["N"]
    dev = D.build_spmm_device(plan.tiles, A, N=N, tc_mode=mode)
    p = DeviceSpmmPlan(dev)
    B = np.random.default_rng(1).standard_normal((A.shape[1], N)).astype(np.float32)
    C = p.run(torch.as_tensor(B, device="cuda"))
    torch.cuda.synchronize()
    ref = S.spmm_fp64(A, B)
    err = S.rel_fro(C.cpu().numpy(), ref)
    print(f"{meta['name']} mode={mode} rel_fro={err:.3e}")
    assert err <= tol
    assert p.error_flag() == 0
    # rows without any nonzero are exactly zero
    empty = np.diff(A.indptr) == 0
    assert np.all(C.cpu().numpy()[empty] == 0)


@pytest.mark.parametrize("path", SPMM_FIXTURES, ids=lambda p: p.split("/")[-1][:-4])
def test_fused_spmm_ell_only_path_is_fp32_exact(path):
    """An ELL-only plan runs entirely in FP32 on CUDA cores (<= 1e-5)."""
    meta, plan, A = _case(path, seed=3)
    if _needs_tc(plan):
        pytest.skip("plan has tensor-core tiles")
    dev = D.build_spmm_device(plan.tiles, A, N=meta["N"])
    p = DeviceSpmmPlan(dev)
    B = np.random.default_rng(2).standard_normal((A.shape[1], meta["N"])).astype(np.float32)
    C = p.run(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert S.rel_fro(C, S.spmm_fp64(A, B)) <= 1e-5


@pytest.mark.parametrize("N", [3, 41, 128, 200, 260])
@pytest.mark.parametrize("name", ["community_1024", "powerlaw_512_ell", "hubblocks_4096"])
def test_fused_spmm_feature_widths(name, N):
    """A plan runs at any feature count: N % 4 != 0 takes the register
    gather path for row tiles, N % 4 == 0 the bulk-copy path; N > 128 spans
    several 128-feature slices."""
    path = [p for p in SPMM_FIXTURES if name in p][0]
    meta, plan, A = _case(path, seed=11)
    if _needs_tc(plan) and not umma_layout_ok():
        pytest.fail("tensor-core layout probe failed; fused kernel not run")
    dev = D.build_spmm_device(plan.tiles, A, N=meta["N"], tc_mode=D.TC_BF16)
    p = DeviceSpmmPlan(dev)
    B = np.random.default_rng(N).standard_normal((A.shape[1], N)).astype(np.float32)
    C = p.run(torch.as_tensor(B, device="cuda")).cpu().numpy()
    tol = 1e-2 if _needs_tc(plan) else 1e-5
    assert S.rel_fro(C, S.spmm_fp64(A, B)) <= tol
    assert p.error_flag() == 0
    empty = np.diff(A.indptr) == 0
    assert np.all(C[empty] == 0)


@pytest.mark.parametrize("dvmode", [1, 2], ids=["tc_dvals", "run_dvals"])
@pytest.mark.parametrize("path", SPMM_FIXTURES, ids=lambda p: p.split("/")[-1][:-4])
def test_dvals_matches_fp64_sddmm(path, dvmode):
    """Value gradients over the forward tiles, the tensor-tile nonzeros on
    the tensor cores (hi + lo bf16) or by row runs: within 1e-5 of float64."""
    meta, plan, A = _case(path, seed=4)
    N = meta["N"]
    dev = D.build_spmm_device(plan.tiles, A, N=N)
    p = DeviceSpmmPlan(dev)
    p.set_dvals_mode(dvmode)
    rng = np.random.default_rng(7)
    dY = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dv = p.dvals(torch.as_tensor(dY, device="cuda"), torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert p.error_flag() == 0
    ref = S.sddmm_fp64(A, dY, B)
    assert S.rel_fro(dv, ref) <= 1e-5


@pytest.mark.parametrize("mode,tol", [(D.TC_BF16, 1e-2), (D.TC_SPLIT_BF16, 1e-5)], ids=["bf16", "split"])
def test_set_values_repacks_in_place(mode, tol):
    path = [p for p in SPMM_FIXTURES if "community_1024" in p][0]
    meta, plan, A = _case(path, seed=5)
    if not umma_layout_ok():
        pytest.fail("tensor-core layout probe failed; fused kernel not run")
    dev = D.build_spmm_device(plan.tiles, A, N=meta["N"], tc_mode=mode)
    p = DeviceSpmmPlan(dev)
    A2 = random_values(A, seed=99)
    p.set_values(torch.as_tensor(A2.data.astype(np.float32), device="cuda"))
    B = np.random.default_rng(3).standard_normal((A.shape[1], meta["N"])).astype(np.float32)
    C = p.run(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert S.rel_fro(C, S.spmm_fp64(A2, B)) <= tol


@pytest.mark.parametrize("N", [1, 3, 16, 41, 64, 128, 200])
def test_csr_kernel_matches_fp64(N):
    from stile_gb300 import synthetic as syn
    A = syn.power_law_rows(4096, 4096, min_len=1, seed=0)
    C = CsrMatrix(A)
    B = np.random.default_rng(N).standard_normal((4096, N)).astype(np.float32)
    out = C.spmm(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert S.rel_fro(out, S.spmm_fp64(A, B)) <= 1e-5


def test_csr_kernel_empty_rows_and_empty_matrix():
    import scipy.sparse as sp
    A = sp.csr_matrix((np.array([2.0]), np.array([3]), np.array([0, 0, 1, 1])), shape=(3, 8))
    B = np.arange(8 * 4, dtype=np.float32).reshape(8, 4)
    out = CsrMatrix(A).spmm(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert np.array_equal(out, np.asarray(A @ B, dtype=np.float32))
    Z = sp.csr_matrix((0, 8))
    assert CsrMatrix(Z).spmm(torch.as_tensor(B, device="cuda")).shape == (0, 4)


@pytest.mark.parametrize("N", [128, 41, 4096])
def test_bf16_dense_operand(N):
    """A bf16 B is read as is (row tiles convert it to fp32, tensor tiles
    feed it to the MMA): against the fp64 product with the same bf16 values,
    the row-tile-only plan is fp32-exact and the hybrid plan is within the
    bf16 tensor-tile tolerance."""
    from stile_gb300 import workloads as W
    from stile_gb300.api import PlanConfig, SpmmOperator
    import torch
    if N == 4096:
        A = W.pruned(False).A
    else:
        A = syn.community_graph(n=8192, target_nnz=90_000, seed=3)
    B = torch.randn((A.shape[1], N), device="cuda").to(torch.bfloat16)
    Bf = B.float().cpu().numpy()
    ref = S.spmm_fp64(A, Bf)
    hyb = SpmmOperator(A, N, PlanConfig(tc_mode=D.TC_BF16))
    assert hyb.device_layout.stats()["tc_ksteps"] > 0
    C = hyb(B).cpu().numpy()
    assert S.rel_fro(C, ref) <= 1e-2
    assert S.rel_fro(C, hyb(B.float()).cpu().numpy()) <= 1e-5   # same products as the fp32 B path
    ell = SpmmOperator(A, N, PlanConfig(tc_mode=D.TC_BF16, only_ELL=True))
    assert S.rel_fro(ell(B).cpu().numpy(), ref) <= 1e-5
    assert hyb.handle.error_flag() == 0 and ell.handle.error_flag() == 0


def test_bf16_dense_operand_needs_bf16_tensor_tiles():
    from stile_gb300.api import PlanConfig, SpmmOperator
    import torch
    A = syn.community_graph(n=4096, target_nnz=40_000, seed=4)
    op = SpmmOperator(A, 64, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    assert op.device_layout.stats()["tc_ksteps"] > 0
    B = torch.randn((A.shape[1], 64), device="cuda").to(torch.bfloat16)
    with pytest.raises(RuntimeError, match="bf16 tensor tiles"):
        op(B)


@pytest.mark.parametrize("N", [41, 128, 200])
def test_tensor_tile_dvals_on_wide_and_ragged_widths(N):
    """The tensor-core value-gradient kernel at N not a multiple of 64 (a
    partial feature chunk, masked loads) and N > 128 (several chunks), on a
    plan with dense tensor tiles; the row-run result is the check."""
    path = [p for p in SPMM_FIXTURES if "community_2048.npz" in p][0]
    meta, plan, A = _case(path, seed=21)
    dev = D.build_spmm_device(plan.tiles, A, N=N)
    p = DeviceSpmmPlan(dev)
    rng = np.random.default_rng(N + 3)
    dY = torch.as_tensor(rng.standard_normal((A.shape[0], N)).astype(np.float32), device="cuda")
    B = torch.as_tensor(rng.standard_normal((A.shape[1], N)).astype(np.float32), device="cuda")
    p.set_dvals_mode(1)
    tc = p.dvals(dY, B).cpu().numpy()
    p.set_dvals_mode(2)
    runs = p.dvals(dY, B).cpu().numpy()
    assert p.error_flag() == 0
    ref = S.sddmm_fp64(A, dY.cpu().numpy(), B.cpu().numpy())
    assert S.rel_fro(tc, ref) <= 1e-5 and S.rel_fro(runs, ref) <= 1e-5
