"""Host-side fault injection at the C ABI: every validation branch of the plan
uploads and of the run entry points rejects a corrupted plan or argument
with STILE_E_INVALID (or STILE_E_UNSUPPORTED) and its message, before any
device call (so these tests need no GPU).  The plans start from a reference
plan of the golden fixtures (tensor-core and ELL tiles) and from a mixed
SDDMM plan, and one array at a time is corrupted."""
import ctypes
import dataclasses
import os

import numpy as np
import pytest

import oracle.semantics as S
from golden_plan import plan_from_fixture
from stile_gb300 import _lib
from stile_gb300 import device as D
from stile_gb300.ops import sddmm_plan_host, spmm_plan_host

HERE = os.path.dirname(os.path.abspath(__file__))
INVALID, UNSUPPORTED = -1, -4


@pytest.fixture(scope="module")
def spmm_dev():
    meta, arr = S.load_fixture(os.path.join(HERE, "golden", "spmm_powerlaw_4096.npz"))
    plan = plan_from_fixture(meta, arr)
    A = S.fixture_matrix(meta, arr)
    dev = D.build_spmm_device(plan.tiles, A, N=meta["N"], tc_mode=D.TC_BF16)
    assert len(dev.tc_cols) and len(dev.ell_kidx)
    # a valid zero-row list (rows the upload may zero) to corrupt below
    return dataclasses.replace(dev, zero_rows=np.array([0, 5], np.int32))


@pytest.fixture(scope="module")
def sddmm_dev():
    meta, arr = S.load_fixture(os.path.join(HERE, "golden", "sddmm_mask_1024.npz"))
    plan = plan_from_fixture(meta, arr)
    A = S.fixture_matrix(meta, arr)
    dev = D.build_sddmm_device(plan.tiles, A.shape, A.nnz)
    assert len(dev.mid_idx) and len(dev.blk_out)
    return dev


def _upload_spmm(dev, tweak_host=None):
    lib = _lib.load()
    h, keep = spmm_plan_host(dev)
    if tweak_host:
        tweak_host(h)
    out = ctypes.c_void_p()
    rc = lib.stile_spmm_plan_upload(ctypes.byref(h), ctypes.byref(out))
    del keep
    return rc, out.value


def _upload_sddmm(dev, tweak_host=None):
    lib = _lib.load()
    h, keep = sddmm_plan_host(dev)
    if tweak_host:
        tweak_host(h)
    out = ctypes.c_void_p()
    rc = lib.stile_sddmm_plan_upload(ctypes.byref(h), ctypes.byref(out))
    del keep
    return rc, out.value


def _set(arr_name, fn):
    """A copy of the device layout with array `arr_name` replaced by fn(copy)."""
    def make(dev):
        a = getattr(dev, arr_name).copy()
        return dataclasses.replace(dev, **{arr_name: fn(a)})
    return make


def _poke(i, v):
    def f(a):
        a.flat[i] = v
        return a
    return f


SPMM_CASES = [
    # (case id, device-layout corruption, host-struct corruption, code, message fragment)
    ("negative_shape", None, lambda h: setattr(h, "M", -1), INVALID, "negative shape"),
    ("negative_count", None, lambda h: setattr(h, "ell_n_slots", -3), INVALID, "negative count"),
    ("unknown_tc_mode", None, lambda h: setattr(h, "tc_mode", 99), UNSUPPORTED, "unknown tensor-tile mode"),
    ("fp8_without_row_scales", None, lambda h: setattr(h, "tc_mode", 3), INVALID, "need tc_row_scale"),
    ("fp8_bad_row_scale", lambda d: dataclasses.replace(d, tc_mode=3, tc_row_scale=np.full(
        len(d.tc_item_flags) * 16, -1.0, np.float32)), None, INVALID, "positive and finite"),
    ("kstep_bytes", None, lambda h: setattr(h, "tc_kstep_bytes", 1024), INVALID, "tc_kstep_bytes"),
    ("missing_tc_array", None, lambda h: setattr(h, "tc_cols", None), INVALID, "missing tensor-tile array"),
    ("tc_kbeg_span", _set("tc_item_kbeg", _poke(-1, 0)), None, INVALID, "does not span the k-steps"),
    ("tc_kbeg_monotone", _set("tc_item_kbeg", lambda a: np.concatenate([a[:1], a[2:3], a[1:2], a[3:]])),
     None, INVALID, "not monotone"),
    ("tc_cols_range", _set("tc_cols", _poke(5, 1 << 20)), None, INVALID, "tc_cols out of range"),
    ("tc_cols_negative", _set("tc_cols", _poke(7, -2)), None, INVALID, "tc_cols out of range"),
    ("tc_out_rows_range", _set("tc_out_rows", _poke(3, 1 << 20)), None, INVALID, "tc_out_rows out of range"),
    ("tc_nnz_id_range", _set("tc_nnz_id", _poke(0, 1 << 30)), None, INVALID, "tc_nnz_id out of range"),
    ("missing_ell_array", None, lambda h: setattr(h, "ell_kidx", None), INVALID, "missing ELL array"),
    ("ell_row0_span", _set("ell_item_row0", _poke(-1, 1)), None, INVALID, "does not span the rows"),
    ("ell_item_K", _set("ell_item_K", _poke(0, 0)), None, INVALID, "bad ELL item shape"),
    ("ell_slots_past_end", _set("ell_item_slot0", _poke(-1, 1 << 28)), None, INVALID, "slots out of range"),
    ("ell_row_len", _set("ell_row_len", _poke(0, 1 << 12)), None, INVALID, "ell_row_len > K"),
    ("ell_kidx_range", _set("ell_kidx", _poke(1, 1 << 20)), None, INVALID, "ell_kidx out of range"),
    ("ell_out_row_range", _set("ell_out_row", _poke(2, -7)), None, INVALID, "ell_out_row out of range"),
    ("ell_nnz_id_range", _set("ell_nnz_id", _poke(4, 1 << 30)), None, INVALID, "ell_nnz_id out of range"),
    ("zero_rows_range", _set("zero_rows", _poke(0, 1 << 20)), None, INVALID, "zero_rows out of range"),
    ("zero_rows_null", None, lambda h: setattr(h, "zero_rows", None), INVALID, "zero_rows out of range"),
]


@pytest.mark.parametrize("case,corrupt,tweak,code,msg", SPMM_CASES, ids=[c[0] for c in SPMM_CASES])
def test_spmm_upload_rejects_corrupted_plan(spmm_dev, case, corrupt, tweak, code, msg):
    dev = corrupt(spmm_dev) if corrupt else spmm_dev
    rc, handle = _upload_spmm(dev, tweak)
    assert rc == code and not handle
    assert msg in _lib.last_error(), _lib.last_error()


def test_spmm_upload_null_arguments():
    lib = _lib.load()
    assert lib.stile_spmm_plan_upload(None, None) == INVALID
    assert "null argument" in _lib.last_error()


SDDMM_CASES = [
    ("negative_count", None, lambda h: setattr(h, "n_1d", -1), INVALID, "negative count"),
    ("missing_1d", None, lambda h: setattr(h, "remap", None), INVALID, "missing 1D array"),
    ("mid_idx_range", _set("mid_idx", _poke(0, 1 << 20)), None, INVALID, "1D index out of range"),
    ("j_idx_range", _set("j_idx", _poke(0, -1)), None, INVALID, "1D index out of range"),
    ("remap_range", _set("remap", _poke(0, 1 << 30)), None, INVALID, "1D index out of range"),
    ("block_too_large", None, lambda h: setattr(h, "bm", 32), UNSUPPORTED, "larger than 16x16"),
    ("missing_block", None, lambda h: setattr(h, "blk_out", None), INVALID, "missing block array"),
    ("blk_indptr_span", _set("blk_indptr", _poke(-1, 0)), None, INVALID, "does not span the entries"),
    ("blk_indptr_order", _set("blk_indptr", lambda a: np.concatenate([a[:1], a[2:3], a[1:2], a[3:]])),
     None, INVALID, "bad blk_indptr"),
    ("blk_i_range", _set("blk_i", _poke(0, 1 << 20)), None, INVALID, "block index out of range"),
    ("blk_dense_pos_range", _set("blk_dense_pos", _poke(0, 256)), None, INVALID, "block index out of range"),
    ("blk_out_range", _set("blk_out", _poke(0, -1)), None, INVALID, "block index out of range"),
]


@pytest.mark.parametrize("case,corrupt,tweak,code,msg", SDDMM_CASES, ids=[c[0] for c in SDDMM_CASES])
def test_sddmm_upload_rejects_corrupted_plan(sddmm_dev, case, corrupt, tweak, code, msg):
    dev = corrupt(sddmm_dev) if corrupt else sddmm_dev
    rc, handle = _upload_sddmm(dev, tweak)
    assert rc == code and not handle
    assert msg in _lib.last_error(), _lib.last_error()


def test_run_entry_points_validate_before_launching():
    """Arguments that fail validation return before any device work; the
    pointers passed are never dereferenced (16-byte aligned dummies)."""
    lib = _lib.load()
    fake = 1 << 20  # an aligned dummy address, never read
    assert lib.stile_spmm_run(None, fake, 128, fake, 128, 128, None) == INVALID
    assert "null plan" in _lib.last_error()
    assert lib.stile_sddmm_run(None, fake, 64, fake, 64, fake, 64, None) == INVALID
    assert lib.stile_spmm_dvals(None, fake, 64, fake, 64, fake, 64, None) == INVALID
    assert lib.stile_spmm_plan_set_wait_policy(None, 10, 1) == INVALID
    assert lib.stile_spmm_plan_set_dvals_mode(None, 1) == INVALID
    assert "null plan" in _lib.last_error()
    assert lib.stile_spmm_backward(None, fake, 64, fake, 64, fake, 64, fake, 64, None) == INVALID
    assert lib.stile_spmm_plan_set_transpose_ids(None, fake, 10, None) == INVALID
    # plain CSR kernel: shape, null arrays, strides, alignment, nnz
    csr = lib.stile_csr_spmm_run
    assert csr(4, 8, fake, fake, fake, None, fake, 64, fake, 64, 0, None) == INVALID
    assert "bad shape" in _lib.last_error()
    assert csr(4, 8, None, fake, fake, None, fake, 64, fake, 64, 64, None) == INVALID
    assert "null CSR array" in _lib.last_error()
    assert csr(4, 8, fake, fake, fake, None, fake, 66, fake, 64, 64, None) == INVALID
    assert "row stride" in _lib.last_error()
    assert csr(4, 8, fake, fake, fake, None, fake + 4, 64, fake, 64, 64, None) == INVALID
    assert "16-byte aligned" in _lib.last_error()
    assert csr(4, 8, fake, fake, fake, None, fake, 64, fake, 32, 64, None) == INVALID
    assert csr(4, -1, fake, fake, fake, None, fake, 64, fake, 64, 64, None) == INVALID
    assert "negative nnz" in _lib.last_error()
    # row softmax and the batched entry points
    assert lib.stile_csr_row_softmax(-1, fake, 4, fake, fake, 1.0, 1, None) == INVALID
    assert lib.stile_csr_row_softmax(4, None, 4, fake, fake, 1.0, 1, None) == INVALID
    assert lib.stile_spmm_values_bytes(None, 2) == INVALID
    assert lib.stile_spmm_run_batched(None, fake, 2, fake, 64, 64, fake, 64, 64, 64, None) == INVALID
