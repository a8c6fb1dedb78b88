"""On-disk plan format and plan cache: a saved and reloaded plan emits and
packs into the same arrays, bit for bit, as the plan that was saved, for the
reference's own selected plans (golden fixtures) and for plans of this
package's search; a cached plan is found again and a plan never loads for a
different pattern."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden_files
from golden_plan import plan_from_fixture
from gpu_util import random_values
import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300 import emit
from stile_gb300 import synthetic as syn
from stile_gb300.cost_model import gb300_model
from stile_gb300.plan_io import PlanCache, load_plan, pattern_key, save_plan
from stile_gb300.planner import search_sddmm, search_spmm


def _same(a, b, where=""):
    if isinstance(a, (list, tuple)):
        assert isinstance(b, (list, tuple)) and len(a) == len(b), where
        for n, (x, y) in enumerate(zip(a, b)):
            _same(x, y, f"{where}[{n}]")
        return
    if hasattr(a, "__dataclass_fields__"):
        for k in a.__dataclass_fields__:
            _same(getattr(a, k), getattr(b, k), f"{where}.{k}")
        return
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        a, b = np.asarray(a), np.asarray(b)
        assert a.dtype == b.dtype and a.shape == b.shape, (where, a.dtype, b.dtype, a.shape, b.shape)
        assert np.array_equal(a, b, equal_nan=a.dtype.kind == "f"), where
        return
    assert a == b, (where, a, b)


def _formats_key(fmts):
    return [(f.template, f.tile_sizes, sorted(f.params.items()), len(f.tiles)) for f in fmts]


def _check_spmm_roundtrip(plan, A, N, path):
    save_plan(plan, path, A=A)
    back = load_plan(path, A=A)
    assert back.op_type == plan.op_type and tuple(back.shape) == tuple(plan.shape)
    assert back.level_num == plan.level_num and back.max_bucket_size == plan.max_bucket_size
    assert back.meta == plan.meta and back.summary() == plan.summary()
    M = A.shape[0]
    f1, a1, s1 = emit.emit_spmm_reference(plan.tiles, M, N)
    f2, a2, s2 = emit.emit_spmm_reference(back.tiles, M, N)
    assert _formats_key(f1) == _formats_key(f2) and tuple(s1) == tuple(s2)
    _same(a1, a2, "emitted")
    for mode in (D.TC_BF16, D.TC_SPLIT_BF16):
        _same(D.build_spmm_device(plan.tiles, A, N=N, tc_mode=mode),
              D.build_spmm_device(back.tiles, A, N=N, tc_mode=mode), "device")
    for t, u in zip(plan.tiles, back.tiles):
        assert tuple(t.tile_pos) == tuple(u.tile_pos) and type(t.tile_pos[-1]) is type(u.tile_pos[-1])
        assert t.pred_cost == u.pred_cost and t.nnz_when_selected == u.nnz_when_selected
        if hasattr(t, "cov_ids"):
            assert np.array_equal(t.cov_ids, u.cov_ids)
    return back


def _check_sddmm_roundtrip(plan, A, path):
    save_plan(plan, path, A=A)
    back = load_plan(path, A=A)
    f1, a1 = emit.emit_sddmm_reference(plan.tiles)
    f2, a2 = emit.emit_sddmm_reference(back.tiles)
    assert _formats_key(f1) == _formats_key(f2)
    _same(a1, a2, "emitted")
    _same(D.build_sddmm_device(plan.tiles, A.shape, A.nnz), D.build_sddmm_device(back.tiles, A.shape, A.nnz),
          "device")
    return back


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_reference_plans_round_trip(path, tmp_path):
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    A = random_values(S.fixture_matrix(meta, arr), seed=3)
    if meta["op"] == "spmm":
        _check_spmm_roundtrip(plan, A, meta["N"], str(tmp_path / "p.npz"))
    else:
        _check_sddmm_roundtrip(plan, A, str(tmp_path / "p.npz"))


@pytest.mark.parametrize("case", ["community", "powerlaw", "pruned"])
def test_searched_spmm_plans_round_trip(case, tmp_path):
    if case == "community":
        A = syn.community_graph(n=4096, target_nnz=40_000, seed=1)
    elif case == "powerlaw":
        A = syn.power_law_rows(2048, 2048, min_len=2, max_len=256, seed=2)
    else:
        A = syn.pruned_weight(384, 256, sparsity=0.8, seed=3)
    A = random_values(A, seed=4)
    plan = search_spmm(A, 64, cost=gb300_model())
    back = _check_spmm_roundtrip(plan, A, 64, str(tmp_path / "p.npz"))
    # the lazily computed block orders are stored only where the tiles read
    for t, u in zip(plan.tiles, back.tiles):
        if t.template == "TensorCore_template":
            order_a, order_b = t.op.blk_k_vals[int(t.tile_pos[0])], u.op.blk_k_vals[int(u.tile_pos[0])]
            assert np.array_equal(order_a[t.k_vals], order_b[u.k_vals])


def test_searched_sddmm_plan_round_trips(tmp_path):
    A = random_values(syn.sddmm_mask(n=2048, target_nnz=30_000, seed=6), seed=7)
    plan = search_sddmm(A, 64, cost=gb300_model(), max_bucket_size=32)
    assert {t.template for t in plan.tiles} >= {"1D_sddmm"}
    _check_sddmm_roundtrip(plan, A, str(tmp_path / "s.npz"))


def test_plan_does_not_load_for_another_pattern(tmp_path):
    A = syn.community_graph(n=1024, target_nnz=8000, seed=1)
    plan = search_spmm(A, 32, cost=gb300_model())
    p = str(tmp_path / "p.npz")
    save_plan(plan, p, A=A)
    B = A.tolil()
    B[0, 1023] = 1.0 if A[0, 1023] == 0 else 0.0
    B = sp.csr_matrix(B)
    B.eliminate_zeros()
    assert pattern_key(B) != pattern_key(A)
    with pytest.raises(ValueError, match="different sparsity pattern"):
        load_plan(p, A=B)
    # same pattern, other values: same key
    assert pattern_key(random_values(A, seed=9)) == pattern_key(A)


def test_cache_hits_misses_and_replaces_bad_files(tmp_path):
    A = syn.community_graph(n=1024, target_nnz=8000, seed=2)
    cost = gb300_model()
    kw = dict(cost=cost, max_bucket_size=None)
    calls = []

    def search():
        calls.append(1)
        return search_spmm(A, 32, **kw)

    cache = PlanCache(str(tmp_path))
    p1, src1 = cache.get_or_search("spmm", A, 32, kw, search)
    p2, src2 = cache.get_or_search("spmm", A, 32, kw, search)
    assert (src1, src2) == ("search", "cache") and len(calls) == 1
    assert p2.summary() == p1.summary()
    # another width, another cost model or another setting is another entry
    cache.get_or_search("spmm", A, 64, kw, search)
    other = gb300_model()
    other.ell_owned = (other.ell_owned[0] * 2, other.ell_owned[1])
    cache.get_or_search("spmm", A, 32, dict(kw, cost=other), search)
    cache.get_or_search("spmm", A, 32, dict(kw, max_bucket_size=16), search)
    assert len(calls) == 4 and cache.hits == 1 and cache.misses == 4
    # a damaged file is searched again and replaced
    path = cache.path("spmm", A, 32, kw)
    with open(path, "wb") as f:
        f.write(b"not a plan")
    _, src = cache.get_or_search("spmm", A, 32, kw, search)
    assert src == "search" and len(calls) == 5
    _, src = cache.get_or_search("spmm", A, 32, kw, search)
    assert src == "cache"


def test_stored_block_order_refuses_unstored_positions(tmp_path):
    A = random_values(syn.community_graph(n=4096, target_nnz=40_000, seed=1), seed=4)
    plan = search_spmm(A, 64, cost=gb300_model())
    p = str(tmp_path / "p.npz")
    save_plan(plan, p)
    back = load_plan(p)
    tc = [t for t in back.tiles if t.template == "TensorCore_template"]
    if not tc:
        pytest.skip("plan has no tensor-core tiles")
    order = tc[0].op.blk_k_vals[int(tc[0].tile_pos[0])]
    stored = set(order.pos.tolist())
    missing = next(k for k in range(len(order)) if k not in stored)
    with pytest.raises(KeyError):
        order[missing]
