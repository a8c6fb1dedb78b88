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
