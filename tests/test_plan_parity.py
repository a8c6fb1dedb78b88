"""The planner (tile generation + greedy/local search + withdraw over the
reference's A100 cost calibration) selects the same plan as the reference on
every golden case: packing both plans gives bit-identical arrays."""
import numpy as np
import pytest

from conftest import golden_files
import oracle.semantics as S
from stile_gb300 import emit
from stile_gb300.planner import search_spmm as plan_spmm


def _switches(meta):
    """The search switches the fixture was made with (the reference's
    TC_k_notsorted and single_level env variables; single_level runs with
    max_level_num 1, as the reference asserts)."""
    single = meta.get("single_level", False)
    return dict(tc_k_notsorted=meta.get("TC_k_notsorted", False), single_level=single,
                max_level_num=1 if single else float("inf"),
                max_avg_cost_diff=meta.get("max_avg_cost_diff", 0.2),
                reorder_k_by_nnz=meta.get("reorder_k_by_nnz", True))


@pytest.mark.parametrize("path", golden_files("spmm"), ids=lambda p: p.split("/")[-1][:-4])
def test_spmm_plan_matches_reference(path):
    meta, arr = S.load_fixture(path)
    A = S.fixture_matrix(meta, arr)
    plan = plan_spmm(A, meta["N"], max_bucket_size=meta["max_bucket_size"], only_TC=meta["only_TC"],
                     only_ELL=meta["only_ELL"], no_withdraw=meta.get("no_withdraw", False), **_switches(meta))
    fm, args, out_shape = emit.emit_spmm_reference(plan.tiles, meta["idx_lens"][0], meta["N"])
    assert list(out_shape) == meta["out_shape"]
    assert [f.template for f in fm] == [f["template"] for f in meta["formats"]]
    assert [len(f.tiles) for f in fm] == [f["n_tiles"] for f in meta["formats"]]
    for a, r in zip(args, S.fixture_args(meta, arr)):
        for x, y in zip(a, r):
            x, y = np.asarray(x), np.asarray(y)
            assert x.shape == y.shape
            assert np.array_equal(x.astype(y.dtype), y)


def test_max_bucket_size_estimate():
    from stile_gb300.planner import estimate_max_bucket_size
    # my_search_formats.py:965-981 with SM_num 108
    assert estimate_max_bucket_size(14687) == 8
    assert estimate_max_bucket_size(160081) == 32
    assert estimate_max_bucket_size(1_000) == 4


@pytest.mark.parametrize("path", golden_files("sddmm"), ids=lambda p: p.split("/")[-1][:-4])
def test_sddmm_plan_matches_reference(path):
    from stile_gb300.planner import plan_sddmm
    meta, arr = S.load_fixture(path)
    A = S.fixture_matrix(meta, arr)
    plan = plan_sddmm(A, meta["N"], max_bucket_size=meta["max_bucket_size"], only_TC=meta["only_TC"],
                      only_ELL=meta["only_ELL"], **_switches(meta))
    fm, args = emit.emit_sddmm_reference(plan.tiles)
    assert [f.template for f in fm] == [f["template"] for f in meta["formats"]]
    assert [len(f.tiles) for f in fm] == [f["n_tiles"] for f in meta["formats"]]
    for a, r in zip(args, S.fixture_args(meta, arr)):
        for x, y in zip(a, r):
            x, y = np.asarray(x), np.asarray(y)
            assert x.shape == y.shape
            assert np.array_equal(x.astype(y.dtype), y)


@pytest.mark.parametrize("name", ["spmm_community_1024_single_level", "spmm_hubblocks_4096_no_withdraw",
                                  "spmm_blockpruned_768x512_knots", "spmm_community_2048_kfirst",
                                  "sddmm_mask_1024_single_level"])
def test_reference_named_facade_selects_the_reference_plan(name, monkeypatch):
    """The reference-named facade, called as the reference's drivers call it
    (switches as arguments and as the single_level / no_withdraw environment
    variables), returns the plan the reference selected."""
    from conftest import GOLDEN
    from stile_gb300.api import Op, greedy_search_use_cost_model_lower_bound, post_process_for_withdraw
    meta, arr = S.load_fixture(f"{GOLDEN}/{name}.npz")
    A = S.fixture_matrix(meta, arr)
    monkeypatch.setenv("single_level", str(meta.get("single_level", False)))
    monkeypatch.setenv("no_withdraw", str(meta.get("no_withdraw", False)))
    M, N, K = meta["idx_lens"]
    op = Op(meta["op"], [0, 1], [2], [M, N, K], None, [A], [A.tocsc()])
    res = greedy_search_use_cost_model_lower_bound(
        op, 16, None, meta["max_bucket_size"], ["A"], ([1], [1], [1]), meta["only_TC"], meta["only_ELL"], 1,
        meta.get("TC_k_notsorted", False), reorder_k_by_nnz=meta.get("reorder_k_by_nnz", True),
        max_level_num=1 if meta.get("single_level", False) else float("inf"),
        max_avg_cost_diff=meta.get("max_avg_cost_diff", 0.2))
    tiles = post_process_for_withdraw(op, *res[:4])
    if meta["op"] == "spmm":
        fm, args, _ = emit.emit_spmm_reference(tiles.tiles, M, N)
    else:
        fm, args = emit.emit_sddmm_reference(tiles.tiles)
    assert [len(f.tiles) for f in fm] == [f["n_tiles"] for f in meta["formats"]]
    for a, r in zip(args, S.fixture_args(meta, arr)):
        for x, y in zip(a, r):
            assert np.array_equal(np.asarray(x).astype(np.asarray(y).dtype), np.asarray(y))
