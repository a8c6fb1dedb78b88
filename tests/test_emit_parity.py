"""The emitter packs the reference's selected plans into arrays that are
bit-identical to what the reference's packer emitted for the same plan
(prepare_inputs_BSPMM / prepare_inputs_BSDDMM)."""
import numpy as np
import pytest

from conftest import golden_files
from golden_plan import plan_from_fixture
import oracle.semantics as S
from stile_gb300 import emit


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_emit_bit_exact(path):
    meta, arr = S.load_fixture(path)
    plan = plan_from_fixture(meta, arr)
    ref_args = S.fixture_args(meta, arr)
    if meta["op"] == "spmm":
        fmts, args, out_shape = emit.emit_spmm_reference(plan.tiles, meta["idx_lens"][0], meta["N"])
        assert list(out_shape) == meta["out_shape"]
    else:
        fmts, args = emit.emit_sddmm_reference(plan.tiles)
    assert [f.template for f in fmts] == [f["template"] for f in meta["formats"]]
    assert [len(f.tiles) for f in fmts] == [f["n_tiles"] for f in meta["formats"]]
    for f, a, r in zip(fmts, args, ref_args):
        assert len(a) == len(r)
        for x, y in zip(a, r):
            x, y = np.asarray(x), np.asarray(y)
            assert x.shape == y.shape, (f.template, x.shape, y.shape)
            if y.dtype.kind in "iu":
                assert x.dtype.kind in "iu"
                assert np.array_equal(x, y)
            else:
                assert np.array_equal(x.astype(np.float32), y)
