"""Public API on the GPU: planned operators, the autograd backward (value
and dense-operand gradients) against FP64 references and FP64 central
finite differences, and the GCN-style induced-subgraph gradient check."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300 import synthetic as syn
from stile_gb300.api import HybridSpMMFunction, PlanConfig, plan_sddmm, plan_spmm

pytestmark = pytest.mark.gpu


def _graph(n=2048, nnz=30000, seed=4):
    return syn.community_graph(n=n, target_nnz=nnz, seed=seed, max_deg=512)


@pytest.mark.parametrize("mode,tol", [(D.TC_BF16, 1e-2), (D.TC_SPLIT_BF16, 1e-5)], ids=["bf16", "split"])
def test_plan_spmm_gb300_cost_model(mode, tol):
    A = _graph()
    op = plan_spmm(A, 128, PlanConfig(tc_mode=mode))
    B = np.random.default_rng(0).standard_normal((A.shape[1], 128)).astype(np.float32)
    C = op(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert S.rel_fro(C, S.spmm_fp64(A, B)) <= tol


def test_autograd_gradients_match_fp64():
    A = _graph(seed=7)
    N = 64
    op = plan_spmm(A, N, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    rng = np.random.default_rng(1)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    vals = torch.as_tensor(A.data.astype(np.float32), device="cuda").requires_grad_(True)
    Bt = torch.as_tensor(B, device="cuda").requires_grad_(True)
    C = HybridSpMMFunction.apply(vals, Bt, op)
    gv, gB = torch.autograd.grad(C, [vals, Bt], grad_outputs=torch.as_tensor(dC, device="cuda"))
    assert S.rel_fro(gv.cpu().numpy(), S.sddmm_fp64(A, dC, B)) <= 1e-5
    assert S.rel_fro(gB.cpu().numpy(), S.spmm_fp64(A.T.tocsr(), dC)) <= 1e-5


def test_autograd_follows_new_values():
    A = _graph(seed=8)
    op = plan_spmm(A, 32, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    B = np.random.default_rng(2).standard_normal((A.shape[1], 32)).astype(np.float32)
    new = np.random.default_rng(3).uniform(-1, 1, A.nnz)
    vals = torch.as_tensor(new.astype(np.float32), device="cuda")
    C = HybridSpMMFunction.apply(vals, torch.as_tensor(B, device="cuda"), op).cpu().numpy()
    A2 = sp.csr_matrix((new, A.indices, A.indptr), shape=A.shape)
    assert S.rel_fro(C, S.spmm_fp64(A2, B)) <= 1e-5


def test_autograd_first_backward_uses_new_values():
    """Plan on A's values, then call the function with other values: the
    first backward builds the transposed plan, and its dB must use the new
    values, not the ones the plan was built from; a second step with yet
    other values (the transposed plan now exists) must follow them too."""
    A = _graph(seed=11)
    N = 64
    op = plan_spmm(A, N, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    rng = np.random.default_rng(12)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    Bt = torch.as_tensor(B, device="cuda").requires_grad_(True)
    dCt = torch.as_tensor(dC, device="cuda")
    for step in range(2):
        new = rng.uniform(-1, 1, A.nnz)
        A2 = sp.csr_matrix((new, A.indices, A.indptr), shape=A.shape)
        vals = torch.as_tensor(new.astype(np.float32), device="cuda").requires_grad_(True)
        C = HybridSpMMFunction.apply(vals, Bt, op)
        gv, gB = torch.autograd.grad(C, [vals, Bt], grad_outputs=dCt)
        assert S.rel_fro(C.detach().cpu().numpy(), S.spmm_fp64(A2, B)) <= 1e-5, step
        assert S.rel_fro(gB.cpu().numpy(), S.spmm_fp64(A2.T.tocsr(), dC)) <= 1e-5, step
        assert S.rel_fro(gv.cpu().numpy(), S.sddmm_fp64(A2, dC, B)) <= 1e-5, step


def test_autograd_reloads_values_of_a_new_tensor_and_after_inplace_update():
    """A values tensor freed and a new one allocated (the caching allocator
    hands back the same block, version 0), and an in-place update of the
    values (an optimizer step): each forward and backward uses the values
    the tensor holds."""
    A = _graph(seed=13)
    N = 32
    op = plan_spmm(A, N, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    rng = np.random.default_rng(14)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    Bt = torch.as_tensor(B, device="cuda").requires_grad_(True)
    dCt = torch.as_tensor(dC, device="cuda")

    def check(vals, ref_vals):
        C = HybridSpMMFunction.apply(vals, Bt, op)
        (gB,) = torch.autograd.grad(C, [Bt], grad_outputs=dCt)
        Ar = sp.csr_matrix((ref_vals, A.indices, A.indptr), shape=A.shape)
        assert S.rel_fro(C.detach().cpu().numpy(), S.spmm_fp64(Ar, B)) <= 1e-5
        assert S.rel_fro(gB.cpu().numpy(), S.spmm_fp64(Ar.T.tocsr(), dC)) <= 1e-5

    v1 = rng.uniform(-1, 1, A.nnz).astype(np.float32)
    vals1 = torch.as_tensor(v1, device="cuda")
    check(vals1, v1.astype(np.float64))
    del vals1
    v2 = rng.uniform(-1, 1, A.nnz).astype(np.float32)
    vals2 = torch.as_tensor(v2, device="cuda")
    check(vals2, v2.astype(np.float64))
    with torch.no_grad():
        vals2.mul_(-2.0)
    check(vals2, -2.0 * v2.astype(np.float64))


def test_gradcheck_induced_subgraph_fp64_central_differences():
    """512-node induced subgraph of the GCN-style graph: the analytic
    gradient of L = <dC, A(vals) @ B> from the GPU backward equals FP64
    central differences of L evaluated with the FP64 oracle."""
    G = syn.gcn_graph(n=8192, target_nnz=120000, seed=3, max_deg=1024)
    nodes = np.sort(np.random.default_rng(0).choice(G.shape[0], 512, replace=False))
    A = G[nodes][:, nodes].tocsr()
    A.sort_indices()
    N = 41
    op = plan_spmm(A, N, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    rng = np.random.default_rng(5)
    B = rng.standard_normal((512, N))
    dC = rng.standard_normal((512, N))
    vals = torch.as_tensor(A.data.astype(np.float32), device="cuda").requires_grad_(True)
    Bt = torch.as_tensor(B.astype(np.float32), device="cuda").requires_grad_(True)
    C = HybridSpMMFunction.apply(vals, Bt, op)
    gv, gB = torch.autograd.grad(C, [vals, Bt], grad_outputs=torch.as_tensor(dC.astype(np.float32), device="cuda"))
    gv, gB = gv.cpu().numpy().astype(np.float64), gB.cpu().numpy().astype(np.float64)

    def loss(v, Bm):
        Av = sp.csr_matrix((v, A.indices, A.indptr), shape=A.shape)
        return float(np.sum(dC * (Av @ Bm)))

    v0 = A.data.astype(np.float64)
    h = 1e-6
    # a directional derivative sums many signed terms, so its error is
    # measured on the scale |g| |d| (Cauchy-Schwarz), tolerance 1e-5
    for seed in range(3):
        d = np.random.default_rng(100 + seed).standard_normal(v0.shape)
        num = (loss(v0 + h * d, B) - loss(v0 - h * d, B)) / (2 * h)
        assert abs(num - gv @ d) <= 1e-5 * np.linalg.norm(gv) * np.linalg.norm(d)
        dBdir = np.random.default_rng(200 + seed).standard_normal(B.shape)
        num = (loss(v0, B + h * dBdir) - loss(v0, B - h * dBdir)) / (2 * h)
        assert abs(num - np.sum(gB * dBdir)) <= 1e-5 * np.linalg.norm(gB) * np.linalg.norm(dBdir)
    # and the full gradients against the FP64 dense references
    assert S.rel_fro(gv, S.sddmm_fp64(A, dC, B)) <= 1e-5
    assert S.rel_fro(gB, S.spmm_fp64(A.T.tocsr(), dC)) <= 1e-5


def test_plan_sddmm_api():
    M = syn.sddmm_mask(n=4096, target_nnz=60000, seed=2, max_len=512)
    sop = plan_sddmm(M, 64)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((M.shape[0], 64)).astype(np.float32)
    Y = rng.standard_normal((M.shape[1], 64)).astype(np.float32)
    out = sop(torch.as_tensor(X, device="cuda"), torch.as_tensor(Y, device="cuda")).cpu().numpy()
    assert S.rel_fro(out, S.sddmm_fp64(M, X, Y)) <= 1e-5


@pytest.mark.parametrize("op_type,batch_num", [("spmm", 1), ("batched_spmm", 3)])
def test_reference_named_facade(op_type, batch_num):
    """The reference's driver sequence; measure_latency checks the result
    (every head of a batched run) against scipy at rtol = atol = 1e-2
    before it times."""
    from stile_gb300.api import (Op, greedy_search_use_cost_model_lower_bound, measure_latency,
                                 measure_seleted_formats, post_process_for_withdraw)
    from stile_gb300.synthetic import power_law_rows
    A = power_law_rows(1024, 1024, min_len=4, seed=1, values="ones")
    B = np.random.default_rng(0).random((1024, 64)).astype(np.float32)
    op = Op("spmm", [0, 1], [2], [1024, 64, 1024], None, [A, B], [A.tocsc()])
    res = greedy_search_use_cost_model_lower_bound(op, 16, None, 8, ["A"], ([1], [1], [1]), False, False, 1,
                                                   False, max_avg_cost_diff=0.2)
    tiles = post_process_for_withdraw(op, *res[:4])
    ms = measure_latency(*measure_seleted_formats(op, op_type, batch_num, tiles, 0, ["A"], 16))
    assert ms > 0


def test_plan_cache_reuses_plans_for_operator_and_transpose(tmp_path):
    """With a cache directory the first operator searches and stores its
    plan (and its transpose's, on the first backward); a second operator over
    the same pattern with other values loads both and computes the same
    products as a fresh search."""
    A = syn.power_law_rows(3000, 2500, min_len=2, max_len=300, seed=5)
    N = 64
    cfg = PlanConfig(tc_mode=D.TC_SPLIT_BF16, cache_dir=str(tmp_path))
    op1 = plan_spmm(A, N, cfg)
    assert op1.plan_source == "search"
    assert op1.transposed[0].plan_source == "search"
    A2 = sp.csr_matrix((np.random.default_rng(6).uniform(-1, 1, A.nnz), A.indices, A.indptr), shape=A.shape)
    op2 = plan_spmm(A2, N, cfg)
    opT, _ = op2.transposed
    assert op2.plan_source == "cache" and opT.plan_source == "cache"
    fresh = plan_spmm(A2, N, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    B = torch.as_tensor(np.random.default_rng(7).standard_normal((A.shape[1], N)).astype(np.float32), device="cuda")
    # same arrays on the device; atomic adds may land in another order
    assert torch.allclose(op2(B), fresh(B), rtol=1e-6, atol=1e-6)
    dC = torch.as_tensor(np.random.default_rng(8).standard_normal((A.shape[0], N)).astype(np.float32), device="cuda")
    assert torch.allclose(opT(dC), fresh.transposed[0](dC), rtol=1e-6, atol=1e-6)
    assert S.rel_fro(opT(dC).cpu().numpy(), S.spmm_fp64(A2.T.tocsr(), dC.cpu().numpy())) <= 1e-5


def test_autograd_with_bf16_operand():
    """B in bf16: the forward reads it as is, dvals = <dC, B> runs on the bf16
    rows, dB = A^T dC comes back in bf16; all against fp64 products of the
    same bf16 values."""
    A = _graph(seed=9)
    N = 128
    op = plan_spmm(A, N, PlanConfig(tc_mode=D.TC_BF16))
    rng = np.random.default_rng(3)
    B = torch.as_tensor(rng.standard_normal((A.shape[1], N)).astype(np.float32), device="cuda").to(torch.bfloat16)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    vals = torch.as_tensor(A.data.astype(np.float32), device="cuda").requires_grad_(True)
    Bt = B.clone().requires_grad_(True)
    C = HybridSpMMFunction.apply(vals, Bt, op)
    assert C.dtype == torch.float32
    gv, gB = torch.autograd.grad(C, [vals, Bt], grad_outputs=torch.as_tensor(dC, device="cuda"))
    assert gB.dtype == torch.bfloat16 and gv.dtype == torch.float32
    Bf = B.float().cpu().numpy()
    assert S.rel_fro(C.detach().cpu().numpy(), S.spmm_fp64(A, Bf)) <= 1e-2
    assert S.rel_fro(gv.cpu().numpy(), S.sddmm_fp64(A, dC, Bf)) <= 1e-5
    assert S.rel_fro(gB.float().cpu().numpy(), S.spmm_fp64(A.T.tocsr(), dC)) <= 1e-2


@pytest.mark.parametrize("N", [64, 128])
@pytest.mark.parametrize("mode", [D.TC_BF16, D.TC_SPLIT_BF16], ids=["bf16", "split"])
@pytest.mark.parametrize("knots", [False, True], ids=["sorted", "column_blocks"])
def test_batched_heads_match_one_head_at_a_time(N, mode, knots):
    """Several value sets on one pattern in one launch per kernel give what
    set_values + a single run give for each head (tensor-core columns
    count-sorted, or in column order: the reference's batched TC_k_notsorted
    kernel)."""
    A = _graph(seed=10)
    op = plan_spmm(A, N, PlanConfig(tc_mode=mode, tc_k_notsorted=knots))
    H = 3
    rng = np.random.default_rng(4)
    vals = torch.as_tensor(rng.uniform(-1, 1, (H, A.nnz)).astype(np.float32), device="cuda")
    B = torch.as_tensor(rng.standard_normal((H, A.shape[1], N)).astype(np.float32), device="cuda")
    C = op.batched(vals, B).cpu().numpy()
    for h in range(H):
        Ah = sp.csr_matrix((vals[h].cpu().numpy().astype(np.float64), A.indices, A.indptr), shape=A.shape)
        ref = S.spmm_fp64(Ah, B[h].cpu().numpy())
        assert S.rel_fro(C[h], ref) <= (1e-2 if mode == D.TC_BF16 else 1e-5)
        op.set_values(vals[h])
        one = op(B[h]).cpu().numpy()
        assert np.allclose(C[h], one, rtol=1e-5, atol=1e-5)
    assert op.handle.error_flag() == 0


@pytest.mark.parametrize("N", [128, 41, 64, 200])
@pytest.mark.parametrize("mode", [D.TC_BF16, D.TC_SPLIT_BF16], ids=["bf16", "split"])
@pytest.mark.parametrize("pattern", ["graph", "rect"])
@pytest.mark.parametrize("dvmode", [1, 2], ids=["tc_dvals", "run_dvals"])
def test_fused_backward_matches_separate_passes_and_fp64(N, mode, pattern, dvmode):
    """stile_spmm_backward: dB = A^T dC and dvals from one pass over the
    transposed plan's row tiles (plus a pass for its tensor tiles: on the
    tensor cores, hi + lo bf16, or by row runs) equal the separate
    transposed product and value-gradient pass, and float64 (dvals within
    1e-5 either way); on a symmetric community graph (the transposed plan
    reuses the forward's) and a rectangular power-law matrix (its own
    plan)."""
    if pattern == "graph":
        A = _graph(seed=15)
    else:
        A = syn.power_law_rows(3000, 2200, min_len=2, max_len=300, seed=16)
    op = plan_spmm(A, N, PlanConfig(tc_mode=mode, backward="fused"))
    op.handle.set_dvals_mode(dvmode)
    op.transposed[0].handle.set_dvals_mode(dvmode)
    rng = np.random.default_rng(17)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    Bt, dCt = torch.as_tensor(B, device="cuda"), torch.as_tensor(dC, device="cuda")
    dB, dv = op.backward(dCt, Bt)
    dv_sep = op.dvals(dCt, Bt)
    opT, _ = op.transposed
    dB_sep = opT(dCt)
    torch.cuda.synchronize()
    assert op.handle.error_flag() == 0 and opT.handle.error_flag() == 0
    if dvmode == 2:
        # the same fp32 arithmetic per nonzero: equal up to summation order
        assert torch.allclose(dv, dv_sep, rtol=1e-5, atol=1e-5)
    assert torch.allclose(dB, dB_sep, rtol=1e-5, atol=1e-5)
    tol = 1e-2 if mode == D.TC_BF16 else 1e-5
    assert S.rel_fro(dv.cpu().numpy(), S.sddmm_fp64(A, dC, B)) <= 1e-5
    assert S.rel_fro(dB.cpu().numpy(), S.spmm_fp64(op.A.T.tocsr(), dC)) <= tol


def test_backward_auto_choice_is_timed_once_per_width_and_correct():
    """backward="auto": the first backward of a width times the fused and the
    separate variant on its operands, keeps the faster for later calls, and
    the result matches float64 either way."""
    A = _graph(seed=18)
    op = plan_spmm(A, 64, PlanConfig(tc_mode=D.TC_SPLIT_BF16))
    rng = np.random.default_rng(19)
    B = rng.standard_normal((A.shape[1], 64)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], 64)).astype(np.float32)
    Bt, dCt = torch.as_tensor(B, device="cuda"), torch.as_tensor(dC, device="cuda")
    for _ in range(2):
        dB, dv = op.backward(dCt, Bt)
        assert op._bwd_choice[64] in ("fused", "separate", "fused_tc", "separate_tc")
        assert S.rel_fro(dv.cpu().numpy(), S.sddmm_fp64(A, dC, B)) <= 1e-5
        assert S.rel_fro(dB.cpu().numpy(), S.spmm_fp64(op.A.T.tocsr(), dC)) <= 1e-5
    assert list(op._bwd_choice) == [64]


def test_csr_path_forward_backward_and_value_refresh():
    """path="csr": the plain CSR kernels run the forward (A), the backward's
    dB (A^T) and the value gradient (entry list), all in fp32 (<= 1e-5), and
    they follow new values loaded through the autograd function."""
    A = _graph(seed=11)
    N = 41
    op = plan_spmm(A, N, PlanConfig(path="csr"))
    rng = np.random.default_rng(5)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    Bd, dCd = torch.as_tensor(B, device="cuda"), torch.as_tensor(dC, device="cuda")
    assert S.rel_fro(op(Bd).cpu().numpy(), S.spmm_fp64(A, B)) <= 1e-5
    dB, dv = op.backward(dCd, Bd)
    assert S.rel_fro(dB.cpu().numpy(), S.spmm_fp64(A.T.tocsr(), dC)) <= 1e-5
    assert S.rel_fro(dv.cpu().numpy(), S.sddmm_fp64(A, dC, B)) <= 1e-5
    new = rng.uniform(-1, 1, A.nnz)
    A2 = sp.csr_matrix((new, A.indices, A.indptr), shape=A.shape)
    vals = torch.as_tensor(new.astype(np.float32), device="cuda").requires_grad_(True)
    Bt = Bd.clone().requires_grad_(True)
    C = HybridSpMMFunction.apply(vals, Bt, op)
    assert S.rel_fro(C.detach().cpu().numpy(), S.spmm_fp64(A2, B)) <= 1e-5
    gv, gB = torch.autograd.grad(C, [vals, Bt], grad_outputs=dCd)
    assert S.rel_fro(gB.cpu().numpy(), S.spmm_fp64(A2.T.tocsr(), dC)) <= 1e-5
    assert S.rel_fro(gv.cpu().numpy(), S.sddmm_fp64(A2, dC, B)) <= 1e-5


@pytest.mark.parametrize("N", [128, 41])
def test_auto_path_times_the_candidates_once_and_stays_correct(N):
    """path="auto": the first forward and backward of a width time the
    hybrid plan against the plain CSR kernels (and, for the forward, a dense
    bf16 GEMM of this small matrix) and keep the fastest; either way the
    results match float64 within the tensor-tile bound, and later calls
    reuse the choice."""
    A = _graph(seed=12)
    op = plan_spmm(A, N, PlanConfig(path="auto"))
    rng = np.random.default_rng(6)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    Bd, dCd = torch.as_tensor(B, device="cuda"), torch.as_tensor(dC, device="cuda")
    for _ in range(2):
        C = op(Bd).cpu().numpy()
        assert S.rel_fro(C, S.spmm_fp64(A, B)) <= 1e-2
        dB, dv = op.backward(dCd, Bd)
        assert S.rel_fro(dB.cpu().numpy(), S.spmm_fp64(A.T.tocsr(), dC)) <= 1e-2
        assert S.rel_fro(dv.cpu().numpy(), S.sddmm_fp64(A, dC, B)) <= 1e-5
    # (a 2048-node graph is small enough for the dense GEMM candidate too)
    assert op._fwd_choice[N] in ("hybrid", "csr", "dense")
    assert op._bwd_choice[N] in ("fused", "separate", "fused_tc", "separate_tc", "csr")
    assert len(op._fwd_choice) == 1 and len(op._bwd_choice) == 1


@pytest.mark.parametrize("bf16", [False, True], ids=["fp32", "bf16"])
def test_sddmm_auto_path(bf16):
    mask = syn.community_graph(n=4096, target_nnz=60000, seed=13, max_deg=256)
    F = 64
    op = plan_sddmm(mask, F, PlanConfig(path="auto", max_bucket_size=32))
    rng = np.random.default_rng(8)
    X = torch.as_tensor(rng.standard_normal((mask.shape[0], F)).astype(np.float32), device="cuda")
    Y = torch.as_tensor(rng.standard_normal((mask.shape[1], F)).astype(np.float32), device="cuda")
    if bf16:
        X, Y = X.to(torch.bfloat16), Y.to(torch.bfloat16)
    out = op(X, Y).cpu().numpy()
    assert op._choice and list(op._choice.values())[0] in ("hybrid", "csr")
    ref = S.sddmm_fp64(sp.csr_matrix(mask), X.float().cpu().numpy(), Y.float().cpu().numpy())
    assert S.rel_fro(out, ref) <= 1e-5


def test_auto_path_on_the_pruned_weight_considers_the_dense_gemm():
    """The pruned weight (3072 x 768 at 90% sparsity, N = 4096, bf16 tiles):
    path="auto" times the hybrid plan, the CSR kernel and a dense bf16 GEMM
    of the zero-filled weight, keeps the fastest, and its forward stays
    within the tensor-tile bound; new values reach whichever path runs."""
    from stile_gb300 import workloads as W
    w = W.pruned(False)
    op = plan_spmm(w.A, w.width, PlanConfig(path="auto"))
    B = torch.as_tensor(w.dense["B"], device="cuda")
    C = op(B).cpu().numpy()
    assert op._fwd_choice[w.width] in ("hybrid", "csr", "dense")
    assert S.rel_fro(C, S.spmm_fp64(op.A, w.dense["B"])) <= 1e-2
    # the dense candidate on its own, and after new values
    Cd = op._dense_forward(B).cpu().numpy()
    assert S.rel_fro(Cd, S.spmm_fp64(op.A, w.dense["B"])) <= 1e-2
    new = np.random.default_rng(23).standard_normal(op.nnz) * 0.02
    op.set_values(torch.as_tensor(new.astype(np.float32), device="cuda"))
    A2 = sp.csr_matrix((new, op.A.indices, op.A.indptr), shape=op.A.shape)
    assert S.rel_fro(op(B).cpu().numpy(), S.spmm_fp64(A2, w.dense["B"])) <= 1e-2
    assert S.rel_fro(op._dense_forward(B).cpu().numpy(), S.spmm_fp64(A2, w.dense["B"])) <= 1e-2


def test_outputs_with_unaligned_row_stride_are_filled():
    """An out / dB tensor whose row stride the kernels cannot write (41
    floats: not a multiple of 4) is computed into a padded buffer and copied
    into the caller's tensor."""
    A = _graph(seed=24)
    N = 41
    op = plan_spmm(A, N, PlanConfig(backward="fused"))
    rng = np.random.default_rng(25)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    Bt, dCt = torch.as_tensor(B, device="cuda"), torch.as_tensor(dC, device="cuda")
    C = torch.empty((A.shape[0], N), device="cuda")
    assert C.stride(0) == N
    r = op(Bt, out=C)
    assert r.data_ptr() == C.data_ptr()
    assert S.rel_fro(C.cpu().numpy(), S.spmm_fp64(A, B)) <= 1e-2
    dB = torch.empty((A.shape[1], N), device="cuda")
    r, dv = op.backward(dCt, Bt, dB)
    assert r.data_ptr() == dB.data_ptr()
    assert S.rel_fro(dB.cpu().numpy(), S.spmm_fp64(op.A.T.tocsr(), dC)) <= 1e-2
    with pytest.raises(ValueError):
        op(Bt, out=torch.empty((A.shape[0], N + 1), device="cuda"))
