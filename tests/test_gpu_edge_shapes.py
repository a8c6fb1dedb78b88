"""The kernels on searched plans of edge-case shapes (empty matrices, one
nonzero, one dense row or column, shapes that are not multiples of 16) and
feature widths below 32, against float64."""
import numpy as np
import pytest
import torch

import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300.api import PlanConfig, SddmmOperator, SpmmOperator
from test_edge_shapes import SHAPES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("knots", [False, True], ids=["sorted", "column_blocks"])
@pytest.mark.parametrize("mode,tol", [(D.TC_BF16, 1e-2), (D.TC_SPLIT_BF16, 1e-5)], ids=["bf16", "split"])
@pytest.mark.parametrize("N", [1, 8, 31])
@pytest.mark.parametrize("name", sorted(SHAPES))
def test_spmm_edge_shapes(name, N, mode, tol, knots):
    A = SHAPES[name]()
    op = SpmmOperator(A, N, PlanConfig(tc_mode=mode, tc_k_notsorted=knots))
    B = np.random.default_rng(2).standard_normal((A.shape[1], N)).astype(np.float32)
    C = op(torch.as_tensor(B, device="cuda")).cpu().numpy()
    torch.cuda.synchronize()
    assert op.handle.error_flag() == 0
    assert C.shape == (A.shape[0], N)
    assert S.rel_fro(C, S.spmm_fp64(A, B)) <= tol


@pytest.mark.parametrize("F", [8, 64])
@pytest.mark.parametrize("name", sorted(SHAPES))
def test_sddmm_edge_shapes(name, F):
    A = SHAPES[name]()
    op = SddmmOperator(A, F)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((A.shape[0], F)).astype(np.float32)
    Y = rng.standard_normal((A.shape[1], F)).astype(np.float32)
    out = op(torch.as_tensor(X, device="cuda"), torch.as_tensor(Y, device="cuda")).cpu().numpy()
    assert out.shape == (A.nnz,)
    assert S.rel_fro(out, S.sddmm_fp64(A, X, Y)) <= 1e-5
