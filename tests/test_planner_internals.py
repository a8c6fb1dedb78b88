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


def test_block_pass_terminates_when_a_whole_row_costs_less_than_its_tiles():
    """A 16-row block whose earlier atomic tiles cost more than owning the
    whole row makes the whole-row option's (withdraw) cost negative.  The
    reference's per-block window best * 1.2 then lies below the best and its
    block loop never ends; the planner applies the sign-aware window of the
    reference's main loop, so the search ends and covers every nonzero."""
    import signal

    from stile_gb300 import synthetic as syn
    from stile_gb300.cost_model import gb300_model
    from stile_gb300.planner import search_spmm

    A = syn.community_graph(n=2048, target_nnz=30000, seed=13, max_deg=512)

    def _timeout(*_):
        raise TimeoutError("format search did not end")
    old = signal.signal(signal.SIGALRM, _timeout)
    signal.alarm(60)
    try:
        plan = search_spmm(A, 32, cost=gb300_model(), max_avg_cost_diff=0.2)
    finally:
        signal.alarm(0)
        signal.signal(signal.SIGALRM, old)
    from stile_gb300 import device as D
    from stile_gb300.ops import _tiles_cover_every_nonzero
    dev = D.build_spmm_device(plan.tiles, A, N=32, tc_mode=D.TC_SPLIT_BF16)
    assert _tiles_cover_every_nonzero(dev)
