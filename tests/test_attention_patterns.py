"""The LogSparse and Strided masks built by stile_gb300.synthetic are the
reference's (oracle/attention.py restates its loops)."""
import numpy as np
import pytest

import oracle.attention as OA
from stile_gb300 import synthetic as syn


@pytest.mark.parametrize("n", [3, 4, 17, 100, 1000])
def test_logsparse_matches_reference_definition(n):
    A = syn.logsparse_pattern(n)
    B = OA.rows_to_csr(OA.logsparse_rows(n), n)
    assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


@pytest.mark.parametrize("n", [4, 17, 100, 1000])
def test_strided_matches_reference_definition(n):
    A = syn.strided_pattern(n)
    B = OA.rows_to_csr(OA.strided_rows(n), n)
    assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


def test_attention_oracle_rows_sum_to_one():
    rng = np.random.default_rng(0)
    A = syn.strided_pattern(64)
    Q, K = rng.standard_normal((2, 1, 64, 8))
    V = np.ones((1, 64, 3))
    out = OA.attention_fp64(A, Q, K, V, 0.5)
    assert np.allclose(out, 1.0)        # probabilities of every row sum to 1
