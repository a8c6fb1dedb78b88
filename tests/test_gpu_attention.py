"""Sparse attention on the GPU against the float64 restatement, on the
reference's LogSparse and Strided masks: the fused one-pass kernel (online
softmax, all heads in one launch) and the three-step path (SDDMM -> row
softmax -> hybrid SpMM)."""
import numpy as np
import pytest
import torch

import oracle.attention as OA
import oracle.semantics as S
from stile_gb300 import _lib
from stile_gb300 import device as D
from stile_gb300 import synthetic as syn
from stile_gb300.api import PlanConfig, SparseAttention
from stile_gb300.ops import _stream

pytestmark = pytest.mark.gpu


def test_row_softmax_kernel():
    A = syn.strided_pattern(500)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((3, A.nnz)).astype(np.float32) * 4
    xt = torch.as_tensor(x, device="cuda")
    out = torch.empty_like(xt)
    ip = torch.as_tensor(A.indptr.astype(np.int32), device="cuda")
    lib = _lib.load()
    _lib.check(lib.stile_csr_row_softmax(A.shape[0], ip.data_ptr(), A.nnz, xt.data_ptr(), out.data_ptr(),
                                         0.25, 3, _stream()), "softmax")
    got = out.cpu().numpy()
    for h in range(3):
        for r in range(A.shape[0]):
            a, b = A.indptr[r], A.indptr[r + 1]
            e = np.exp(0.25 * x[h, a:b].astype(np.float64) - 0.25 * x[h, a:b].max())
            assert np.allclose(got[h, a:b], e / e.sum(), rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("kind", ["logsparse", "strided"])
@pytest.mark.parametrize("mode,tol", [(D.TC_BF16, 1e-2), (D.TC_SPLIT_BF16, 1e-5)], ids=["bf16", "split"])
def test_sparse_attention_matches_fp64(kind, mode, tol):
    n, H, F = 2048, 2, 64
    A = syn.logsparse_pattern(n) if kind == "logsparse" else syn.strided_pattern(n)
    rng = np.random.default_rng(2)
    Q, K, V = (rng.standard_normal((H, n, F)).astype(np.float32) for _ in range(3))
    att = SparseAttention(A, F, cfg=PlanConfig(tc_mode=mode), fused=False)
    out = att(*(torch.as_tensor(x, device="cuda") for x in (Q, K, V))).cpu().numpy()
    ref = OA.attention_fp64(A, Q, K, V, 1.0 / np.sqrt(F))
    assert S.rel_fro(out, ref) <= tol


@pytest.mark.parametrize("kind", ["logsparse", "strided"])
@pytest.mark.parametrize("F,Fv,H", [(64, 64, 2), (128, 128, 3), (41, 24, 1), (16, 100, 2)])
def test_fused_sparse_attention_matches_fp64(kind, F, Fv, H):
    """The fused kernel (fp32 throughout, online softmax) within 1e-5 of
    float64 on widths that fill 128-feature groups and on ragged ones, and a
    row without entries gives zeros."""
    n = 1500
    A = syn.logsparse_pattern(n) if kind == "logsparse" else syn.strided_pattern(n)
    A = A.tolil()
    A[7, :] = 0          # an empty row
    A = A.tocsr()
    A.eliminate_zeros()
    rng = np.random.default_rng(3)
    Q = rng.standard_normal((H, n, F)).astype(np.float32)
    K = rng.standard_normal((H, n, F)).astype(np.float32)
    V = rng.standard_normal((H, n, Fv)).astype(np.float32)
    att = SparseAttention(A, F, Fv)
    assert att.fused
    out = att(*(torch.as_tensor(x, device="cuda") for x in (Q, K, V))).cpu().numpy()
    ref = OA.attention_fp64(A, Q, K, V, 1.0 / np.sqrt(F))
    assert np.all(out[:, 7] == 0)
    assert S.rel_fro(out, ref) <= 1e-5
