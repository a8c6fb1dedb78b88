"""Pin the CPU oracle: executing the reference-emitted arrays of every golden
plan with the oracle's restatement of the fused-kernel arithmetic must give
scipy's float64 A @ B (SpMM) / masked X Y^T (SDDMM)."""
import numpy as np
import pytest

from conftest import golden_files
import oracle.semantics as S


@pytest.mark.parametrize("path", golden_files("spmm"), ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_spmm_matches_fp64(path):
    meta, arr = S.load_fixture(path)
    A = S.fixture_matrix(meta, arr)
    args = S.fixture_args(meta, arr)
    B = np.random.default_rng(0).standard_normal((A.shape[1], meta["N"]))
    C, conflicts = S.spmm_from_arrays(meta["formats"], args, B, meta["out_shape"])
    M = A.shape[0]
    assert S.rel_fro(C[:M, :meta["N"]], S.spmm_fp64(A, B)) < 1e-13
    # owned rows below M are written once (sentinel row M may be written many times);
    # the only tolerated exception is the zero store of ELL padding rows
    assert all(r >= M for r in conflicts) or meta["name"] == "spmm_powerlaw_512_ell"


@pytest.mark.parametrize("path", golden_files("sddmm"), ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_sddmm_matches_fp64(path):
    meta, arr = S.load_fixture(path)
    A = S.fixture_matrix(meta, arr)
    args = S.fixture_args(meta, arr)
    rng = np.random.default_rng(1)
    X = rng.standard_normal((A.shape[0], meta["N"]))
    Y = rng.standard_normal((A.shape[1], meta["N"]))
    out = S.sddmm_from_arrays(meta["formats"], args, X, Y, A.nnz)
    assert S.rel_fro(out, S.sddmm_fp64(A, X, Y)) < 1e-13


def test_ell_padding_hazard_is_detected():
    """The reference packs padding rows of the last ELL tile with the tile's
    last output row; under plain stores those rows write zeros into a real
    row.  The oracle sees it; the device layout marks such rows no-write."""
    path = [p for p in golden_files("spmm_powerlaw_512_ell")][0]
    meta, arr = S.load_fixture(path)
    args = S.fixture_args(meta, arr)
    B = np.ones((meta["idx_lens"][2], meta["N"]))
    _, conflicts = S.spmm_from_arrays(meta["formats"], args, B, meta["out_shape"])
    assert any(r < meta["idx_lens"][0] for r in conflicts)
