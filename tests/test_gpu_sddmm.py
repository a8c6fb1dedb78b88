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
