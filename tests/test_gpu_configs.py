"""Parity at the full sizes of the five benchmark configurations
(stile_gb300.workloads): every product of the forward and backward against
the float64 oracle, at the tolerance of the path (fp32 path <= 1e-5, bf16
tensor tiles <= 1e-2 relative Frobenius), and the SDDMM operator on the
2M-nonzero mask.  Value gradients of the large cases are checked on a seeded
sample of 200k entries."""
import numpy as np
import pytest
import torch

import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300 import workloads as W
from stile_gb300.api import HybridSpMMFunction, PlanConfig, SddmmOperator, SpmmOperator

pytestmark = pytest.mark.gpu


def _spmm_products(w, tc_mode, **cfg):
    op = SpmmOperator(w.A, w.width, PlanConfig(tc_mode=tc_mode, **cfg))
    B = torch.as_tensor(w.dense["B"], device="cuda")
    dC = torch.as_tensor(w.dense["dC"], device="cuda")
    C = op(B)
    opT, _ = op.transposed
    dB = opT(dC)
    dv = op.dvals(dC, B)
    torch.cuda.synchronize()
    assert op.handle.error_flag() == 0 and opT.handle.error_flag() == 0
    return op, C.cpu().numpy(), dB.cpu().numpy(), dv.cpu().numpy()


def _check_spmm(w, tc_mode, tol, **cfg):
    op, C, dB, dv = _spmm_products(w, tc_mode, **cfg)
    A = op.A
    assert S.rel_fro(C, S.spmm_fp64(A, w.dense["B"])) <= tol
    assert S.rel_fro(dB, S.spmm_fp64(A.T.tocsr(), w.dense["dC"])) <= tol
    ids, ref = W.sddmm_fp64_sample(A, w.dense["dC"], w.dense["B"])
    assert S.rel_fro(dv[ids], ref) <= 1e-5      # value gradients run in fp32
    return op


@pytest.mark.parametrize("name", ["plain", "plain_min10"])
def test_config1_plain_spmm_fp32_path(name):
    w = W.BY_NAME[name]()
    _check_spmm(w, D.TC_SPLIT_BF16, 1e-5)


@pytest.mark.parametrize("name", ["pruned", "pruned_t"])
def test_config3_pruned_weight_bf16_tiles(name):
    w = W.BY_NAME[name]()
    op = _check_spmm(w, D.TC_BF16, 1e-2)
    # the block-pruned half of the weight goes to the tensor cores
    assert op.device_layout.stats()["tc_ksteps"] > 0


@pytest.mark.parametrize("name", ["pruned", "pruned_t"])
def test_config3_pruned_weight_column_blocks(name):
    """Tensor-core tiles as 16x16 blocks on the column grid (TC_k_notsorted):
    every tensor-core k-step reads 16 consecutive columns starting at a
    multiple of 16, and the products match float64."""
    w = W.BY_NAME[name]()
    op = _check_spmm(w, D.TC_BF16, 1e-2, tc_k_notsorted=True)
    cols = op.device_layout.tc_cols.astype(np.int64).reshape(-1, 16)
    assert len(cols) > 0
    assert np.all(cols[:, 0] % 16 == 0)
    assert np.all(cols == np.minimum(cols[:, :1] + np.arange(16), w.A.shape[1] - 1))


def test_config3_pruned_weight_fp32_path():
    w = W.pruned(False)
    _check_spmm(w, D.TC_SPLIT_BF16, 1e-5)


@pytest.fixture(scope="module")
def sddmm_config():
    w = W.sddmm()
    return w, SddmmOperator(w.A, w.width)


def test_config4_sddmm_mask(sddmm_config):
    w, op = sddmm_config
    X = torch.as_tensor(w.dense["X"], device="cuda")
    Y = torch.as_tensor(w.dense["Y"], device="cuda")
    out = op(X, Y).cpu().numpy()
    ids, ref = W.sddmm_fp64_sample(w.A, w.dense["X"], w.dense["Y"], n_sample=w.A.nnz)
    assert len(ids) == w.A.nnz
    assert S.rel_fro(out, ref) <= 1e-5


def test_config4_sddmm_mask_bf16(sddmm_config):
    """X and Y in bf16 (the configuration's second precision): read as is,
    products and sums in fp32, so against the fp64 product of the same bf16
    values the result is fp32-exact."""
    w, op = sddmm_config
    X = torch.as_tensor(w.dense["X"], device="cuda").to(torch.bfloat16)
    Y = torch.as_tensor(w.dense["Y"], device="cuda").to(torch.bfloat16)
    out = op(X, Y).cpu().numpy()
    ids, ref = W.sddmm_fp64_sample(w.A, X.float().cpu().numpy(), Y.float().cpu().numpy(), n_sample=w.A.nnz)
    assert S.rel_fro(out, ref) <= 1e-5


def test_config2_hybrid_graph():
    """The bench graph (169,343 nodes, 1.17M nonzeros, N = 128): forward and
    dB within the bf16 tolerance, dvals (fp32) on every nonzero."""
    w = W.graph()
    op, C, dB, dv = _spmm_products(w, D.TC_BF16)
    A = op.A
    assert S.rel_fro(C, S.spmm_fp64(A, w.dense["B"])) <= 1e-2
    assert S.rel_fro(dB, S.spmm_fp64(A.T.tocsr(), w.dense["dC"])) <= 1e-2
    assert S.rel_fro(dv, S.sddmm_fp64(A, w.dense["dC"], w.dense["B"])) <= 1e-5
    assert op.device_layout.stats()["tc_ksteps"] > 0 and op.device_layout.stats()["ell_slots"] > 0


@pytest.fixture(scope="module")
def gcn_graph_ops():
    """The GCN graph (232,965 nodes, ~11.4M nonzeros) and its operators for
    the two layer widths, 128 and 41 (one plan each)."""
    w = W.gcn(128)
    assert w.A.nnz > 11_000_000
    op128 = SpmmOperator(w.A, 128, PlanConfig(tc_mode=D.TC_BF16))
    op41 = SpmmOperator(w.A, 41, PlanConfig(tc_mode=D.TC_BF16))
    return w, op128, op41


def _check_op(op, B_np, dC_np, tol):
    B = torch.as_tensor(B_np, device="cuda")
    dC = torch.as_tensor(dC_np, device="cuda")
    C = op(B).cpu().numpy()
    opT, _ = op.transposed
    dB = opT(dC).cpu().numpy()
    dv = op.dvals(dC, B).cpu().numpy()
    torch.cuda.synchronize()
    assert op.handle.error_flag() == 0 and opT.handle.error_flag() == 0
    A = op.A
    assert S.rel_fro(C, S.spmm_fp64(A, B_np)) <= tol
    assert S.rel_fro(dB, S.spmm_fp64(A.T.tocsr(), dC_np)) <= tol
    ids, ref = W.sddmm_fp64_sample(A, dC_np, B_np)
    assert S.rel_fro(dv[ids], ref) <= 1e-5


def test_config5_gcn_layer_full_graph(gcn_graph_ops):
    w, op128, _ = gcn_graph_ops
    _check_op(op128, w.dense["B"], w.dense["dC"], 1e-2)
    # symmetric pattern: the transposed operator reuses the forward plan
    assert op128.transposed[0].plan is op128.plan


def test_config5_gcn_layer2_N41(gcn_graph_ops):
    """The second layer's width, 41 features (not a multiple of the 128-feature
    tensor-core slice nor of the 16-byte vector): operands with a padded
    row stride of 44."""
    w, _, op41 = gcn_graph_ops
    rng = np.random.default_rng(41)
    n = w.A.shape[0]
    B = rng.standard_normal((n, 41)).astype(np.float32)
    dC = rng.standard_normal((n, 41)).astype(np.float32)
    _check_op(op41, B, dC, 1e-2)


def _gcn2_fp64(A, X, W1, W2, G, mask):
    """float64 forward and gradients of L = <G, A relu(A X W1) W2> with respect
    to W1, W2 and A's values (one value set shared by both layers).  The ReLU
    mask is given (the GPU's H1 > 0): an entry of H1 within rounding of zero
    may change sign, and its gradient then differs by the whole value, which
    says nothing about the products' accuracy."""
    A = A.astype(np.float64)
    XW1 = X @ W1
    H1 = A @ XW1
    Z1 = np.where(mask, H1, 0.0)
    XW2 = Z1 @ W2
    H2 = A @ XW2
    AT = A.T.tocsr()
    dXW2 = AT @ G
    dW2 = Z1.T @ dXW2
    dH1 = (dXW2 @ W2.T) * mask
    dXW1 = AT @ dH1
    dW1 = X.T @ dXW1
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    dvals = (np.einsum("ij,ij->i", G[rows], XW2[A.indices]) + np.einsum("ij,ij->i", dH1[rows], XW1[A.indices]))
    return H2, dW1, dW2, dvals


@pytest.mark.parametrize("where", ["induced_512", "full_graph"])
def test_config5_two_layer_gcn_step(gcn_graph_ops, where):
    """The two-layer GCN step, 602 -> 128 -> 41, through HybridSpMMFunction:
    the output and the gradients of W1, W2 and of the shared edge values
    against float64, on the 512-node induced subgraph (fp32 path, 1e-5) and
    on the full graph (bf16 tensor tiles, 1e-2)."""
    from stile_gb300.gcn import TwoLayerGCN
    w, op128, op41 = gcn_graph_ops
    if where == "induced_512":
        # 512 consecutive nodes: their planted 16x16 communities stay inside
        # the induced subgraph (920 edges), random nodes keep almost none
        nodes = np.arange(100_000, 100_512)
        A = w.A[nodes][:, nodes].tocsr()
        A.sort_indices()
        assert A.nnz > 0
        cfg = PlanConfig(tc_mode=D.TC_SPLIT_BF16)
        ops, tol = None, 1e-5
    else:
        A, cfg, ops, tol = op128.A, None, (op128, op41), 1e-2
    n = A.shape[0]
    rng = np.random.default_rng(5)
    X = rng.standard_normal((n, 602)).astype(np.float32)
    W1 = (rng.standard_normal((602, 128)) / np.sqrt(602)).astype(np.float32)
    W2 = (rng.standard_normal((128, 41)) / np.sqrt(128)).astype(np.float32)
    G = rng.standard_normal((n, 41)).astype(np.float32)
    model = TwoLayerGCN(A, torch.as_tensor(W1, device="cuda"), torch.as_tensor(W2, device="cuda"), cfg, ops=ops)
    Xt = torch.as_tensor(X, device="cuda")
    # the model's forward, step by step so that H1 (its ReLU mask) is seen
    H1 = HybridSpMMFunction.apply(model.vals, model.lin1(Xt), model.op1)
    H2 = HybridSpMMFunction.apply(model.vals, model.lin2(torch.relu(H1)), model.op2)
    gW1, gW2, gv = torch.autograd.grad(H2, [model.lin1.weight, model.lin2.weight, model.vals],
                                       grad_outputs=torch.as_tensor(G, device="cuda"))
    torch.cuda.synchronize()
    mask = H1.detach().cpu().numpy() > 0
    rH2, rW1, rW2, rdv = _gcn2_fp64(A, X.astype(np.float64), W1.astype(np.float64), W2.astype(np.float64),
                                    G.astype(np.float64), mask)
    assert S.rel_fro(H2.detach().cpu().numpy(), rH2) <= tol
    assert S.rel_fro(gW2.cpu().numpy(), rW2) <= tol
    assert S.rel_fro(gW1.cpu().numpy(), rW1) <= tol
    assert S.rel_fro(gv.cpu().numpy(), rdv) <= tol
