"""FP8 e4m3 tensor tiles (STILE_TC_FP8) on the GPU.

The tile values are stored as e4m3 of value / (row scale), the row scale
being the tile row's largest |value| / 448; B is converted in the kernel to
e4m3 of B / s_x with s_x = max|B| / 448 from an amax pass; the MMA is
kind::f8f6f4 with fp32 accumulation and the epilogue multiplies by
s_x * row scale.  Row tiles stay fp32.

Two checks: against a float64 emulation of exactly that arithmetic (the same
e4m3 rounding of both operands), which pins layouts, byte order and scales
within fp32 accumulation error; and against the exact float64 product,
which measures what e4m3 costs (stated in the assertion's bound)."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import torch

import oracle.semantics as S
from golden_plan import plan_from_fixture
from stile_gb300 import device as D
from stile_gb300 import workloads as W
from stile_gb300.api import PlanConfig, SpmmOperator
from stile_gb300.ops import DeviceSpmmPlan

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def fp8_emulation(dev, A, B):
    """float64 C of the fp8 path: row tiles exact, tensor tiles with the
    e4m3-rounded values and the e4m3-rounded B (same scales as the kernel)."""
    A = sp.csr_matrix(A, dtype=np.float64)
    B = np.asarray(B, np.float32)
    amax = np.float32(np.abs(B).max())
    # as the kernel: x * (448 / amax) in fp32, then e4m3; undone by amax / 448
    xinv = np.float32(D.E4M3_MAX) / amax if amax > 0 else np.float32(0.0)
    _, Bq = D.to_e4m3(B * xinv)
    Bq = Bq.astype(np.float64) * (float(amax) / D.E4M3_MAX)
    nks = len(dev.tc_cols) // 16
    item_of = np.repeat(np.arange(len(dev.tc_item_kbeg) - 1), np.diff(dev.tc_item_kbeg))
    s = dev.tc_row_scale.reshape(-1, 16)[item_of].astype(np.float64)          # [nks, 16]
    _, q = D.to_e4m3((dev.tc_values_f32 / s[:, :, None]).astype(np.float32))
    wq = q.astype(np.float64) * s[:, :, None]                                   # [nks, 16, 16]
    ids = dev.tc_nnz_id.reshape(nks, 16, 16)
    live = ids >= 0
    tc_ids = ids[live]
    vals = A.data.copy()
    is_tc = np.zeros(A.nnz, bool)
    is_tc[tc_ids] = True
    A_ell = sp.csr_matrix((np.where(is_tc, 0.0, vals), A.indices, A.indptr), shape=A.shape)
    tcv = np.zeros(A.nnz)
    tcv[tc_ids] = wq[live]
    A_tc = sp.csr_matrix((tcv, A.indices, A.indptr), shape=A.shape)
    return A_ell @ B.astype(np.float64) + A_tc @ Bq


@pytest.mark.parametrize("name", ["spmm_pruned_256x192.npz", "spmm_community_2048.npz", "spmm_mixed_2048.npz",
                                  "spmm_blockpruned_768x512_knots.npz"])
@pytest.mark.parametrize("N", [64, 128, 41])
def test_fp8_tiles_match_their_float64_emulation(name, N):
    meta, arr = S.load_fixture(os.path.join(HERE, "golden", name))
    plan = plan_from_fixture(meta, arr)
    A = S.fixture_matrix(meta, arr)
    A.data = np.random.default_rng(1).standard_normal(A.nnz) * 0.02
    dev = D.build_spmm_device(plan.tiles, A, N=N, tc_mode=D.TC_FP8)
    assert len(dev.tc_cols) > 0
    p = DeviceSpmmPlan(dev)
    B = np.random.default_rng(2).standard_normal((A.shape[1], N)).astype(np.float32)
    C = p.run(torch.as_tensor(B, device="cuda"))
    torch.cuda.synchronize()
    assert p.error_flag() == 0
    ref = fp8_emulation(dev, A, B)
    assert S.rel_fro(C.cpu().numpy(), ref) <= 1e-5


def test_fp8_pruned_weight_config3_error_and_emulation():
    """The pruned weight (3072 x 768 at 90% sparsity, N = 4096): the fp8
    tiles equal their emulation within fp32 accumulation error, and against
    the exact product the whole forward is within 5e-2 relative Frobenius
    (e4m3 keeps 3 mantissa bits; the bf16 tiles give 1.5e-3 here)."""
    w = W.pruned(False)
    op = SpmmOperator(w.A, w.width, PlanConfig(tc_mode=D.TC_FP8))
    B = w.dense["B"]
    C = op(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert op.handle.error_flag() == 0
    assert S.rel_fro(C, fp8_emulation(op.device_layout, op.A, B)) <= 1e-5
    err = S.rel_fro(C, S.spmm_fp64(op.A, B))
    print(f"fp8 tiles, pruned weight: rel. Frobenius {err:.3e}")
    assert err <= 5e-2


def test_fp8_plan_rejects_value_refresh_and_bf16_operands():
    meta, arr = S.load_fixture(os.path.join(HERE, "golden", "spmm_pruned_256x192.npz"))
    plan = plan_from_fixture(meta, arr)
    A = S.fixture_matrix(meta, arr)
    dev = D.build_spmm_device(plan.tiles, A, N=64, tc_mode=D.TC_FP8)
    p = DeviceSpmmPlan(dev)
    with pytest.raises(RuntimeError, match="fp8"):
        p.set_values(torch.zeros(A.nnz, device="cuda"))
    with pytest.raises(RuntimeError, match="bf16"):
        p.run(torch.zeros((A.shape[1], 64), device="cuda", dtype=torch.bfloat16))
