"""Searched plans on edge-case shapes: empty matrices, a single nonzero,
one dense row or column, shapes that are not multiples of 16 and feature
widths below 32.  The reference pads its inputs to full blocks and uses
N >= 32, so none of these occur in its runs; here every one must plan in a
bounded time, pack, and compute the float64 product."""
import numpy as np
import pytest
import scipy.sparse as sp

from device_exec import spmm_device_exec
import oracle.semantics as S
from stile_gb300 import device as D
from stile_gb300 import emit
from stile_gb300.planner import search_sddmm, search_spmm

SHAPES = {
    "empty_100x80": lambda: sp.csr_matrix((100, 80)),
    "one_entry_10x9": lambda: sp.csr_matrix(([2.0], ([5], [7])), shape=(10, 9)),
    "dense_row_1x300": lambda: sp.csr_matrix(np.ones((1, 300))),
    "dense_col_300x1": lambda: sp.csr_matrix(np.ones((300, 1))),
    "dense_17x33": lambda: sp.csr_matrix(np.random.default_rng(0).standard_normal((17, 33))),
    "random_50x70": lambda: sp.random(50, 70, density=0.3, format="csr", random_state=1),
}


@pytest.mark.timeout(60)
@pytest.mark.parametrize("knots", [False, True], ids=["sorted", "column_blocks"])
@pytest.mark.parametrize("N", [1, 8, 31, 64])
@pytest.mark.parametrize("name", sorted(SHAPES))
def test_spmm_plan_edge_shapes(name, N, knots):
    A = SHAPES[name]()
    plan = search_spmm(A, N, tc_k_notsorted=knots)
    dev = D.build_spmm_device(plan.tiles, A, N=N)
    B = np.random.default_rng(2).standard_normal((A.shape[1], N))
    C = spmm_device_exec(dev, B)
    assert C.shape == (A.shape[0], N)
    assert not np.isnan(C).any()
    assert np.allclose(C, S.spmm_fp64(A, B), rtol=1e-6, atol=1e-6)


@pytest.mark.timeout(60)
@pytest.mark.parametrize("knots", [False, True], ids=["sorted", "column_blocks"])
@pytest.mark.parametrize("F", [8, 64])
@pytest.mark.parametrize("name", sorted(SHAPES))
def test_sddmm_plan_edge_shapes(name, F, knots):
    A = SHAPES[name]()
    plan = search_sddmm(A, F, tc_k_notsorted=knots)
    fm, args = emit.emit_sddmm_reference(plan.tiles)
    D.build_sddmm_device(plan.tiles, A.shape, A.nnz, emitted=(fm, args))
    rng = np.random.default_rng(3)
    X = rng.standard_normal((A.shape[0], F))
    Y = rng.standard_normal((A.shape[1], F))
    fmts = [{"template": f.template, "tile_sizes": f.tile_sizes, "params": f.params} for f in fm]
    out = S.sddmm_from_arrays(fmts, args, X, Y, A.nnz)
    assert np.allclose(out, S.sddmm_fp64(A, X, Y), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("kind", ["spmm", "sddmm"])
@pytest.mark.parametrize("name", sorted(SHAPES))
def test_plan_file_round_trip_edge_shapes(name, kind, tmp_path):
    """Plans of the edge-case shapes save and load to the same packed arrays."""
    from stile_gb300 import plan_io
    A = SHAPES[name]()
    plan = search_spmm(A, 8, tc_k_notsorted=True) if kind == "spmm" else search_sddmm(A, 8)
    path = str(tmp_path / "plan.npz")
    plan_io.save_plan(plan, path, A=A)
    back = plan_io.load_plan(path, A=A)
    if kind == "spmm":
        a, b = (emit.emit_spmm_reference(p.tiles, A.shape[0], 8)[1] for p in (plan, back))
    else:
        a, b = (emit.emit_sddmm_reference(p.tiles)[1] for p in (plan, back))
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert all(np.array_equal(np.asarray(u), np.asarray(v)) for u, v in zip(x, y))
