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
from stile_gb300.api import PlanConfig, SddmmOperator, SpmmOperator

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


def test_config5_gcn_layer_full_graph():
    w = W.gcn(128)
    assert w.A.nnz > 11_000_000
    op = _check_spmm(w, D.TC_BF16, 1e-2)
    # symmetric pattern: the transposed operator reuses the forward plan
    assert op.transposed[0].plan is op.plan
