"""stile_csr_spmm_run_noalloc: plain CSR SpMM that allocates nothing.

Some callers must not allocate device memory: their memory belongs to
another allocator (a host framework's caching pool, an arena handed out up
front), and a cudaMalloc of their own may also synchronise the device.  The
regular CSR entry point wants a group -> first-row map in a buffer the
caller allocates; the no-allocation entry point builds that map in scratch
memory compiled into the library (1 MiB per GPU, so at most 16,777,216
nonzeros).  Its output must equal the regular entry point's, call after
call, although every call reuses the same scratch.

This file is collected last, so a run that stops at the first failure has
run every other test before this one.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from stile_gb300 import _lib
from stile_gb300 import synthetic as syn

MAX_NNZ = (1 << 18) * 64
TOL = 1e-5  # fp32 CUDA-core path


def _group_rows(A, group_nnz):
    starts = np.arange(0, max(A.nnz, 1), group_nnz, dtype=np.int64)
    rows = np.searchsorted(A.indptr, starts, side="right") - 1
    return np.minimum(rows, max(A.shape[0] - 1, 0)).astype(np.int32)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_noalloc_rejects_inputs_beyond_its_scratch():
    """More nonzeros than the scratch covers is an argument error, reported
    before anything touches the GPU."""
    lib = _lib.load()
    rc = lib.stile_csr_spmm_run_noalloc(16, MAX_NNZ + 1, None, None, None, None, 16, None, 16, 16, None)
    assert rc == -1
    msg = _lib.last_error()
    assert "16777216" in msg and "no-allocation" in msg


@pytest.mark.gpu
def test_noalloc_matches_csr_entry_point_on_consecutive_calls():
    import torch
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    gn = int(lib.stile_csr_group_nnz())
    # two different matrices in a row: the second call finds the first
    # call's map in the shared scratch and must not depend on it
    A1 = syn.power_law_rows(4096, 4096, min_len=1, seed=3)
    A2 = sp.csr_matrix(syn.power_law_rows(3000, 5000, min_len=1, seed=4))
    keep = sp.diags((np.arange(3000) % 7 != 0).astype(np.float64))  # every 7th row empty
    A2 = sp.csr_matrix(keep @ A2)
    A2.eliminate_zeros()
    for A, N in [(A1, 64), (A2, 41)]:
        A = sp.csr_matrix(A, dtype=np.float32)
        A.sort_indices()
        M, K = A.shape
        indptr = torch.as_tensor(A.indptr.astype(np.int32), device="cuda")
        indices = torch.as_tensor(A.indices.astype(np.int32), device="cuda")
        vals = torch.as_tensor(A.data.astype(np.float32), device="cuda")
        rows = torch.as_tensor(_group_rows(A, gn), device="cuda")
        ld = (N + 3) // 4 * 4
        B = torch.zeros((K, ld), device="cuda")
        B[:, :N] = torch.as_tensor(np.random.default_rng(N).standard_normal((K, N)).astype(np.float32), device="cuda")
        C_ref = torch.full((M, ld), float("nan"), device="cuda")
        C_new = torch.full((M, ld), float("nan"), device="cuda")
        rc = lib.stile_csr_spmm_run(M, A.nnz, indptr.data_ptr(), indices.data_ptr(), vals.data_ptr(),
                                    rows.data_ptr(), B.data_ptr(), ld, C_ref.data_ptr(), ld, N, stream)
        assert rc == 0, _lib.last_error()
        rc = lib.stile_csr_spmm_run_noalloc(M, A.nnz, indptr.data_ptr(), indices.data_ptr(), vals.data_ptr(),
                                            B.data_ptr(), ld, C_new.data_ptr(), ld, N, stream)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        ref = C_ref[:, :N].cpu().numpy()
        new = C_new[:, :N].cpu().numpy()
        assert np.isfinite(new).all()
        assert _rel(new, ref) <= TOL
        exact = (A.astype(np.float64) @ B[:, :N].cpu().numpy().astype(np.float64))
        assert _rel(new, exact) <= TOL
