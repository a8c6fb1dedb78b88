"""Failure detection on the GPU without a fault: the tensor-core kernel's
bounded waits.  With a short poll limit and the stall test on, the MMA
issuer waits on a barrier that nothing arrives on; that wait and then every
other role's wait run out, the kernel returns, and the plan's error flag
reads non-zero.  The context stays usable: the next run with the default
policy is correct and leaves the flag clear."""
import numpy as np
import pytest
import torch

import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300 import synthetic as syn
from stile_gb300.api import PlanConfig, plan_spmm

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [D.TC_BF16, D.TC_SPLIT_BF16], ids=["bf16", "split"])
def test_wait_that_runs_out_sets_the_error_flag_and_the_next_run_is_correct(mode):
    A = syn.community_graph(n=4096, target_nnz=60000, seed=21, max_deg=512)
    N = 128
    op = plan_spmm(A, N, PlanConfig(tc_mode=mode))
    assert op.device_layout.stats()["tc_ksteps"] > 0
    B_np = np.random.default_rng(22).standard_normal((A.shape[1], N)).astype(np.float32)
    B = torch.as_tensor(B_np, device="cuda")
    h = op.handle
    assert h.error_flag() == 0
    h.set_wait_policy(polls=1000, stall_test=True)
    op(B)
    torch.cuda.synchronize()          # the run returns
    assert h.error_flag() != 0
    assert h.error_flag() == 0        # reading the flag clears it
    h.set_wait_policy(0, False)
    C = op(B)
    torch.cuda.synchronize()
    assert h.error_flag() == 0
    tol = 1e-2 if mode == D.TC_BF16 else 1e-5
    assert S.rel_fro(C.cpu().numpy(), S.spmm_fp64(A, B_np)) <= tol


def test_short_poll_limit_without_a_stall_returns():
    """A poll limit of 1 on a normal run: waits may give up (the flag then
    says so and the output is undefined) or all succeed (the output is then
    correct); either way the call returns and the next default run is
    correct."""
    A = syn.community_graph(n=4096, target_nnz=60000, seed=23, max_deg=512)
    N = 64
    op = plan_spmm(A, N, PlanConfig(tc_mode=D.TC_BF16))
    B_np = np.random.default_rng(24).standard_normal((A.shape[1], N)).astype(np.float32)
    B = torch.as_tensor(B_np, device="cuda")
    ref = S.spmm_fp64(A, B_np)
    op.handle.set_wait_policy(polls=1)
    C = op(B)
    torch.cuda.synchronize()
    if op.handle.error_flag() == 0:
        assert S.rel_fro(C.cpu().numpy(), ref) <= 1e-2
    op.handle.set_wait_policy(0)
    C = op(B)
    torch.cuda.synchronize()
    assert op.handle.error_flag() == 0
    assert S.rel_fro(C.cpu().numpy(), ref) <= 1e-2
