"""Planner building blocks against direct restatements: the distinct-column
count of every ELL tile position (the B footprint the cost model reads) and
the folded-row layout of an ELL operator."""
import numpy as np
import pytest

from stile_gb300 import synthetic as syn
from stile_gb300.planner import EllOp, Pattern


def _op(seed, mbs):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(20, 500))
    A = syn.power_law_rows(n, n, min_len=1, max_len=min(200, n), seed=seed)
    pat = Pattern(A)
    ids = np.sort(rng.choice(pat.nnz, max(1, pat.nnz // 2), replace=False))
    return pat, ids, EllOp(pat, ids, mbs, 0)


@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("mbs", [4, 32])
def test_ell_tile_distinct_columns(seed, mbs):
    """k_is: distinct columns of the entries in each I-row segment, plus the
    fill column 0 when the segment holds fewer than I*K entries and column 0
    is not among them (for power-of-two and other heights I)."""
    pat, ids, op = _op(seed, mbs)
    K = 4
    for I in (1, 2, 3, 5, 8, 16, 64, 256):
        n_t = -(-op.n_folded // I)
        pos = np.arange(n_t)
        seg = op.frow // I
        distinct = np.array([len(np.unique(op.cols[seg == s])) for s in range(n_t)])
        has0 = np.array([np.any(op.cols[seg == s] == 0) for s in range(n_t)])
        size = np.array([np.count_nonzero(seg == s) for s in range(n_t)])
        ref = distinct + ((size < I * K) & ~has0)
        assert np.array_equal(op.k_is(I, K, pos), ref)


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("mbs", [4, 32])
def test_ell_folded_rows(seed, mbs):
    """Rows in order of decreasing length (stable), each cut into folds of
    mbs entries; every entry of the subset appears once, in its row's column
    order, and each folded row belongs to the right original row."""
    pat, ids, op = _op(seed, mbs)
    assert np.array_equal(np.sort(op.ids), ids)
    assert np.array_equal(np.diff(op.indptr), np.bincount(op.frow, minlength=op.n_folded))
    assert np.all(np.diff(op.indptr) <= mbs)
    rows = pat.row_of[op.ids]
    assert np.array_equal(op.i_perm[op.hyb_new_rows[op.frow]], rows)
    rn = np.bincount(rows, minlength=pat.M)
    assert np.array_equal(np.sort(-rn[op.i_perm], kind="stable"), -rn[op.i_perm])
    for r in np.unique(rows):
        assert np.array_equal(op.cols[rows == r], np.sort(pat.indices[ids[pat.row_of[ids] == r]]))
