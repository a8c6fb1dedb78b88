"""tf32 tensor tiles (STILE_TC_TF32) on the GPU.

The tile values are stored rounded to tf32 (to nearest, ties away from
zero); B's fp32 rows are copied into shared memory as they are and the
tensor core reads them as tf32, i.e. with the low 13 mantissa bits
dropped; products accumulate in fp32.  Row tiles stay fp32.

Checked against a float64 emulation of exactly that arithmetic (pins the
operand layouts and the rounding within fp32 accumulation error), and
against the exact float64 product (what tf32 costs, stated in the bound)."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import oracle.semantics as S
from conftest import golden_files
from golden_plan import plan_from_fixture
from gpu_util import random_values
from stile_gb300 import device as D
from stile_gb300.ops import DeviceSpmmPlan

pytestmark = pytest.mark.gpu


def tf32_trunc(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32) & np.uint32(0xFFFFE000)
    return b.view(np.float32)


def tf32_emulation(dev, A, B):
    """float64 C of the tf32 path: row tiles exact, tensor tiles with the
    rounded values and B's rows truncated to tf32."""
    A = sp.csr_matrix(A, dtype=np.float64)
    B = np.asarray(B, np.float32)
    nks = len(dev.tc_cols) // 16
    ids = dev.tc_nnz_id.reshape(nks, 16, 16)
    live = ids >= 0
    tc_ids = ids[live]
    is_tc = np.zeros(A.nnz, bool)
    is_tc[tc_ids] = True
    A_ell = sp.csr_matrix((np.where(is_tc, 0.0, A.data), A.indices, A.indptr), shape=A.shape)
    tcv = np.zeros(A.nnz)
    tcv[tc_ids] = D.to_tf32(dev.tc_values_f32)[live].astype(np.float64)
    A_tc = sp.csr_matrix((tcv, A.indices, A.indptr), shape=A.shape)
    return A_ell @ B.astype(np.float64) + A_tc @ tf32_trunc(B).astype(np.float64)


@pytest.mark.parametrize("N", [64, 128, 41, 200])
@pytest.mark.parametrize("name", ["community_1024", "mixed_2048", "hubblocks_4096", "pruned_256x192"])
def test_tf32_tiles_match_their_float64_emulation(name, N):
    path = [p for p in golden_files("spmm") if name in p][0]
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    A = random_values(S.fixture_matrix(meta, arr), seed=2)
    dev = D.build_spmm_device(plan.tiles, A, N=N, tc_mode=D.TC_TF32)
    p = DeviceSpmmPlan(dev)
    B = np.random.default_rng(N).standard_normal((A.shape[1], N)).astype(np.float32)
    C = p.run(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert p.error_flag() == 0
    if len(dev.tc_cols):
        assert S.rel_fro(C, tf32_emulation(dev, A, B)) <= 1e-5
    # tf32 keeps 10 explicit mantissa bits: well inside the tensor-tile bound
    assert S.rel_fro(C, S.spmm_fp64(A, B)) <= 2e-3
    empty = np.diff(A.indptr) == 0
    assert np.all(C[empty] == 0)


def test_tf32_batched_heads_and_fused_backward():
    """Value sets packed per head and the fused backward run with tf32 tiles
    (the transposed plan in the same mode)."""
    from stile_gb300.api import PlanConfig, SpmmOperator
    path = [p for p in golden_files("spmm") if "community_1024" in p][0]
    meta, arr = S.load_fixture(path)
    A = random_values(S.fixture_matrix(meta, arr), seed=6)
    N = 64
    op = SpmmOperator(A, N, PlanConfig(tc_mode=D.TC_TF32, backward="fused"))
    rng = np.random.default_rng(4)
    B = rng.standard_normal((A.shape[1], N)).astype(np.float32)
    dC = rng.standard_normal((A.shape[0], N)).astype(np.float32)
    dB, dv = op.backward(torch.as_tensor(dC, device="cuda"), torch.as_tensor(B, device="cuda"))
    assert S.rel_fro(dB.cpu().numpy(), S.spmm_fp64(sp.csr_matrix(A).T.tocsr(), dC)) <= 2e-3
    assert S.rel_fro(dv.cpu().numpy(), S.sddmm_fp64(sp.csr_matrix(A), dC, B)) <= 1e-5
    H = 3
    vals = np.stack([random_values(A, seed=10 + h).data for h in range(H)]).astype(np.float32)
    Bh = rng.standard_normal((H, A.shape[1], N)).astype(np.float32)
    Ch = op.batched(torch.as_tensor(vals, device="cuda"), torch.as_tensor(Bh, device="cuda")).cpu().numpy()
    for h in range(H):
        Ah = sp.csr_matrix((vals[h].astype(np.float64), op.A.indices, op.A.indptr), shape=op.A.shape)
        assert S.rel_fro(Ch[h], S.spmm_fp64(Ah, Bh[h])) <= 2e-3
