"""Torch-facing wrappers over the C ABI (device memory, streams and the
autograd plumbing; the computation is in the sm_103a kernels)."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .device import SddmmDevice, SpmmDevice


def _ptr(a: np.ndarray, ct=ctypes.c_int32):
    return a.ctypes.data_as(ctypes.POINTER(ct)) if a is not None and a.size else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _require_cuda(t: torch.Tensor, name: str):
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor (there is no CPU path)")


def dense_operand(x: torch.Tensor, name="B"):
    """fp32, CUDA, row-major with a row stride that is a multiple of 4 and
    a 16-byte aligned base; copies only when needed."""
    _require_cuda(x, name)
    if x.dtype != torch.float32:
        x = x.float()
    if x.dim() != 2:
        raise ValueError(f"{name} must be 2-D")
    rows, cols = x.shape
    ld = x.stride(0)
    ok = x.stride(1) == 1 and ld >= cols and ld % 4 == 0 and x.data_ptr() % 16 == 0
    if not ok:
        ldp = (cols + 3) // 4 * 4
        buf = torch.zeros((rows, ldp), dtype=torch.float32, device=x.device)
        buf[:, :cols] = x
        x = buf[:, :cols]
        ld = ldp
    return x, ld


def dense_operand_bf16(x: torch.Tensor, name="B"):
    """bf16, CUDA, row-major with a row stride that is a multiple of 8 and a
    16-byte aligned base; copies only when needed."""
    _require_cuda(x, name)
    if x.dtype != torch.bfloat16:
        raise TypeError(f"{name} must be bfloat16")
    if x.dim() != 2:
        raise ValueError(f"{name} must be 2-D")
    rows, cols = x.shape
    ld = x.stride(0)
    ok = x.stride(1) == 1 and ld >= cols and ld % 8 == 0 and x.data_ptr() % 16 == 0
    if not ok:
        ldp = (cols + 7) // 8 * 8
        buf = torch.zeros((rows, ldp), dtype=torch.bfloat16, device=x.device)
        buf[:, :cols] = x
        x = buf[:, :cols]
        ld = ldp
    return x, ld


def new_output(rows, cols, device):
    ldp = (cols + 3) // 4 * 4
    buf = torch.empty((rows, ldp), dtype=torch.float32, device=device)
    return buf[:, :cols], ldp


def output_operand(out: torch.Tensor | None, rows: int, cols: int, device):
    """(buffer the kernels write, its row stride, the caller's out or None):
    the caller's fp32 [rows, cols] out when the kernels can write it in place
    (row stride a multiple of 4, 16-byte aligned base), else a padded buffer
    whose result finish_output copies into out."""
    if out is None:
        buf, ld = new_output(rows, cols, device)
        return buf, ld, None
    _require_cuda(out, "out")
    if out.dtype != torch.float32 or tuple(out.shape) != (rows, cols):
        raise ValueError(f"out must be a float32 tensor of shape ({rows}, {cols})")
    ld = out.stride(0)
    if out.stride(1) == 1 and ld >= cols and ld % 4 == 0 and out.data_ptr() % 16 == 0:
        return out, ld, None
    buf, ld = new_output(rows, cols, device)
    return buf, ld, out


def finish_output(buf: torch.Tensor, target: torch.Tensor | None) -> torch.Tensor:
    if target is None:
        return buf
    target.copy_(buf)
    return target


class PackedValues:
    """H value sets of one plan packed on the device (pack_values)."""

    def __init__(self, buf, off, heads):
        self.buf, self.heads = buf, heads
        self.ptr = buf.data_ptr() + off


def spmm_plan_host(dev: SpmmDevice):
    """(StileSpmmPlanHost over the arrays of ``dev``, the arrays it points
    into): the host side of stile_spmm_plan_upload.  The arrays must stay
    alive until the upload returns."""
    h = _lib.SpmmPlanHost()
    h.M, h.K, h.nnz = dev.M, dev.K, dev.nnz
    h.tc_mode = dev.tc_mode
    h.tc_n_items = len(dev.tc_item_flags)
    h.tc_n_ksteps = len(dev.tc_cols) // 16
    keep = [dev.tc_item_kbeg, dev.tc_item_flags, dev.tc_out_rows, dev.tc_cols, dev.tc_vals,
            dev.tc_nnz_id, dev.ell_item_row0, dev.ell_item_K, dev.ell_item_slot0,
            dev.ell_item_flags, dev.ell_out_row, dev.ell_row_len, dev.ell_vals, dev.ell_kidx,
            dev.ell_nnz_id, dev.zero_rows]
    h.tc_item_kbeg = _ptr(dev.tc_item_kbeg)
    h.tc_item_flags = _ptr(dev.tc_item_flags)
    h.tc_out_rows = _ptr(dev.tc_out_rows)
    h.tc_cols = _ptr(dev.tc_cols)
    h.tc_vals = dev.tc_vals.ctypes.data if dev.tc_vals.size else None
    h.tc_kstep_bytes = dev.tc_kstep_bytes
    h.tc_nnz_id = _ptr(dev.tc_nnz_id)
    h.ell_n_items = len(dev.ell_item_K)
    h.ell_n_rows = len(dev.ell_out_row)
    h.ell_n_slots = len(dev.ell_kidx)
    h.ell_item_row0 = _ptr(dev.ell_item_row0)
    h.ell_item_K = _ptr(dev.ell_item_K)
    h.ell_item_slot0 = _ptr(dev.ell_item_slot0)
    h.ell_item_flags = _ptr(dev.ell_item_flags)
    h.ell_out_row = _ptr(dev.ell_out_row)
    h.ell_row_len = _ptr(dev.ell_row_len)
    h.ell_vals = _ptr(dev.ell_vals, ctypes.c_float)
    h.ell_kidx = _ptr(dev.ell_kidx)
    h.ell_nnz_id = _ptr(dev.ell_nnz_id)
    h.n_zero_rows = len(dev.zero_rows)
    h.zero_rows = _ptr(dev.zero_rows)
    keep.append(dev.tc_row_scale)
    h.tc_row_scale = _ptr(dev.tc_row_scale, ctypes.c_float)
    return h, keep


def sddmm_plan_host(dev: SddmmDevice):
    """(StileSddmmPlanHost over the arrays of ``dev``, the arrays)."""
    h = _lib.SddmmPlanHost()
    h.M, h.K, h.nnz = dev.M, dev.K, dev.nnz
    h.n_1d = len(dev.mid_idx)
    h.mid_idx, h.j_idx, h.remap = _ptr(dev.mid_idx), _ptr(dev.j_idx), _ptr(dev.remap)
    h.n_blk = len(dev.blk_indptr) - 1
    h.bm, h.bn = dev.bm, dev.bn
    h.n_blk_nnz = len(dev.blk_out)
    h.blk_i, h.blk_j = _ptr(dev.blk_i), _ptr(dev.blk_j)
    h.blk_indptr = _ptr(dev.blk_indptr)
    h.blk_dense_pos, h.blk_out = _ptr(dev.blk_dense_pos), _ptr(dev.blk_out)
    keep = [dev.mid_idx, dev.j_idx, dev.remap, dev.blk_i, dev.blk_j, dev.blk_indptr, dev.blk_dense_pos, dev.blk_out]
    return h, keep


def _tiles_cover_every_nonzero(dev: SpmmDevice) -> bool:
    """True when the written tile entries (tensor-core rows with an output
    row, live ELL slots of rows with an output row) hold every nonzero id
    exactly once: the value gradient then writes all of dvals."""
    ids = []
    if len(dev.tc_cols):
        nks = len(dev.tc_cols) // 16
        item = np.repeat(np.arange(len(dev.tc_item_flags)), np.diff(dev.tc_item_kbeg))
        rows_ok = dev.tc_out_rows.reshape(-1, 16)[item] >= 0              # [nks, 16]
        nid = dev.tc_nnz_id.reshape(nks, 16, 16)
        ids.append(nid[rows_ok[:, :, None] & (nid >= 0)])
    if len(dev.ell_kidx):
        K = dev.ell_item_K
        nrows = np.diff(dev.ell_item_row0)
        row_k = np.repeat(K, nrows)
        row_s0 = np.repeat(dev.ell_item_slot0, nrows) + (np.arange(len(row_k)) - np.repeat(dev.ell_item_row0[:-1],
                                                                                            nrows)) * row_k
        live = (dev.ell_out_row >= 0) & (dev.ell_row_len > 0)
        lens = dev.ell_row_len[live].astype(np.int64)
        starts = row_s0[live].astype(np.int64)
        slot = np.repeat(starts - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens) + np.arange(lens.sum())
        nid = dev.ell_nnz_id[slot]
        ids.append(nid[nid >= 0])
    if not ids:
        return dev.nnz == 0
    ids = np.concatenate(ids).astype(np.int64)
    return len(ids) == dev.nnz and bool(np.all(np.bincount(ids, minlength=dev.nnz) == 1))


class DeviceSpmmPlan:
    """A packed SpMM plan resident on the current CUDA device."""

    def __init__(self, dev: SpmmDevice):
        self.lib = _lib.load()
        self.dev = dev
        self.M, self.K, self.nnz = dev.M, dev.K, dev.nnz
        h, self._keep = spmm_plan_host(dev)
        handle = ctypes.c_void_p()
        _lib.check(self.lib.stile_spmm_plan_upload(ctypes.byref(h), ctypes.byref(handle)),
                   "stile_spmm_plan_upload")
        self.handle = handle
        self._dvals_cover_all = _tiles_cover_every_nonzero(dev)
        # tensor tiles with nonzero ids: their value gradients can run on the
        # tensor cores (stile_spmm_plan_set_dvals_mode)
        self.has_tensor_tiles = len(dev.tc_cols) > 0 and len(dev.tc_nnz_id) > 0

    def run(self, B: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """C = A @ B in fp32; B is fp32 or bf16 (a bf16 B is read as is:
        half the gathered bytes, fp32 accumulation)."""
        bf16 = B.dtype == torch.bfloat16
        B, ldb = dense_operand_bf16(B, "B") if bf16 else dense_operand(B, "B")
        if B.shape[0] != self.K:
            raise ValueError(f"B has {B.shape[0]} rows, the plan has K={self.K}")
        N = B.shape[1]
        out, ldc, target = output_operand(out, self.M, N, B.device)
        fn = self.lib.stile_spmm_run_bf16 if bf16 else self.lib.stile_spmm_run
        _lib.check(fn(self.handle, B.data_ptr(), ldb, out.data_ptr(), ldc, N, _stream()),
                   "stile_spmm_run_bf16" if bf16 else "stile_spmm_run")
        return finish_output(out, target)

    def pack_values(self, vals: torch.Tensor) -> "PackedValues":
        """Pack H value sets (vals [H, nnz], CSR order) for run_batched."""
        _require_cuda(vals, "vals")
        vals = vals.float().contiguous()
        if vals.dim() != 2 or vals.shape[1] != self.nnz:
            raise ValueError("vals must be [heads, nnz]")
        H = vals.shape[0]
        nbytes = int(self.lib.stile_spmm_values_bytes(self.handle, H))
        if nbytes < 0:
            _lib.check(nbytes, "stile_spmm_values_bytes")
        buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=vals.device)
        off = (-buf.data_ptr()) % 256
        _lib.check(self.lib.stile_spmm_values_pack(self.handle, vals.data_ptr(), H, buf.data_ptr() + off, _stream()),
                   "stile_spmm_values_pack")
        return PackedValues(buf, off, H)

    def run_batched(self, packed: "PackedValues", B: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """C[h] = A_h @ B[h] for the H value sets of ``packed``; B [H, K, N]
        fp32; one launch of each kernel for all heads."""
        _require_cuda(B, "B")
        B = B.float()
        H, K, N = B.shape
        if H != packed.heads or K != self.K:
            raise ValueError("B must be [heads, K, N] for the packed heads")
        ldb = (N + 3) // 4 * 4
        if B.stride() != (K * ldb, ldb, 1) or B.data_ptr() % 16:
            buf = torch.zeros((H, K, ldb), dtype=torch.float32, device=B.device)
            buf[:, :, :N] = B
            B = buf
        if out is None:
            out = torch.empty((H, self.M, ldb), dtype=torch.float32, device=B.device)[:, :, :N]
        if out.stride(2) != 1 or out.stride(1) % 4 or out.stride(0) % 4 or out.data_ptr() % 16:
            raise ValueError("out rows must be 16-byte aligned with strides that are multiples of 4")
        _lib.check(self.lib.stile_spmm_run_batched(self.handle, packed.ptr, H, B.data_ptr(), B.stride(1),
                                                   B.stride(0), out.data_ptr(), out.stride(1), out.stride(0), N,
                                                   _stream()), "stile_spmm_run_batched")
        return out

    def dvals(self, dY: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
        """dvals[t] = <dY[row(t)], B[col(t)]> (fp32); B fp32 or bf16."""
        dY, lddy = dense_operand(dY, "dY")
        bf16 = B.dtype == torch.bfloat16
        B, ldb = dense_operand_bf16(B, "B") if bf16 else dense_operand(B, "B")
        # the value gradient writes every nonzero the tiles hold
        alloc = torch.empty if self._dvals_cover_all else torch.zeros
        out = alloc(self.nnz, dtype=torch.float32, device=B.device)
        fn = self.lib.stile_spmm_dvals_bf16 if bf16 else self.lib.stile_spmm_dvals
        _lib.check(fn(self.handle, dY.data_ptr(), lddy, B.data_ptr(), ldb, out.data_ptr(), B.shape[1], _stream()),
                   "stile_spmm_dvals_bf16" if bf16 else "stile_spmm_dvals")
        return out

    def set_transpose_ids(self, perm: torch.Tensor):
        """This plan is the transposed operator of a forward plan: perm[t] is
        the forward's nonzero that this plan's nonzero t is (device int32)."""
        perm = perm.to(torch.int32).contiguous()
        if perm.numel() != self.nnz:
            raise ValueError("perm must have one entry per nonzero")
        self._perm = perm
        _lib.check(self.lib.stile_spmm_plan_set_transpose_ids(self.handle, perm.data_ptr(), self.nnz, _stream()),
                   "stile_spmm_plan_set_transpose_ids")

    def backward(self, dC: torch.Tensor, B: torch.Tensor, dB: torch.Tensor | None = None):
        """(dB, dvals) of the forward C = A @ B whose transposed plan this is:
        dB = A^T @ dC and dvals = <dC[row], B[col]> over A's nonzeros (forward
        numbering), from one pass over this plan's row tiles
        (stile_spmm_backward); fp32 operands."""
        dC, lddc = dense_operand(dC, "dC")
        B, ldb = dense_operand(B, "B")
        N = dC.shape[1]
        dB, lddb, target = output_operand(dB, self.M, N, dC.device)
        alloc = torch.empty if self._dvals_cover_all else torch.zeros
        dvals = alloc(self.nnz, dtype=torch.float32, device=dC.device)
        _lib.check(self.lib.stile_spmm_backward(self.handle, dC.data_ptr(), lddc, B.data_ptr(), ldb, dB.data_ptr(),
                                                lddb, dvals.data_ptr(), N, _stream()), "stile_spmm_backward")
        return finish_output(dB, target), dvals

    def set_values(self, vals: torch.Tensor):
        _require_cuda(vals, "vals")
        vals = vals.float().contiguous()
        if vals.numel() != self.nnz:
            raise ValueError("vals must have one entry per nonzero")
        _lib.check(self.lib.stile_spmm_plan_set_values(self.handle, vals.data_ptr(), _stream()),
                   "stile_spmm_plan_set_values")

    def set_wait_policy(self, polls: int = 0, stall_test: bool = False):
        """Poll limit of the tensor-core kernel's pipeline waits (0: the
        default) and the failure-detection stall test
        (stile_spmm_plan_set_wait_policy)."""
        _lib.check(self.lib.stile_spmm_plan_set_wait_policy(self.handle, int(polls), 1 if stall_test else 0),
                   "stile_spmm_plan_set_wait_policy")

    def set_dvals_mode(self, mode: int):
        """Value gradients of the tensor-tile nonzeros: 0 automatic, 1 on the
        tensor cores, 2 by the row runs (stile_spmm_plan_set_dvals_mode)."""
        _lib.check(self.lib.stile_spmm_plan_set_dvals_mode(self.handle, int(mode)), "stile_spmm_plan_set_dvals_mode")

    def error_flag(self) -> int:
        f = ctypes.c_int32(0)
        _lib.check(self.lib.stile_spmm_plan_error_flag(self.handle, _stream(), ctypes.byref(f)),
                   "stile_spmm_plan_error_flag")
        return int(f.value)

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.stile_spmm_plan_free(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceSddmmPlan:
    def __init__(self, dev: SddmmDevice):
        self.lib = _lib.load()
        self.dev = dev
        self.M, self.K, self.nnz = dev.M, dev.K, dev.nnz
        h, self._keep = sddmm_plan_host(dev)
        handle = ctypes.c_void_p()
        _lib.check(self.lib.stile_sddmm_plan_upload(ctypes.byref(h), ctypes.byref(handle)),
                   "stile_sddmm_plan_upload")
        self.handle = handle

    def error_flag(self) -> int:
        f = ctypes.c_int32(0)
        _lib.check(self.lib.stile_sddmm_plan_error_flag(self.handle, _stream(), ctypes.byref(f)),
                   "stile_sddmm_plan_error_flag")
        return int(f.value)

    def run(self, X: torch.Tensor, Y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """out[t] = <X[row(t)], Y[col(t)]> in fp32; X and Y both bf16 are read
        as is, any other mix is computed from fp32 copies."""
        bf16 = X.dtype == torch.bfloat16 and Y.dtype == torch.bfloat16
        if bf16:
            X, ldx = dense_operand_bf16(X, "X")
            Y, ldy = dense_operand_bf16(Y, "Y")
        else:
            X, ldx = dense_operand(X, "X")
            Y, ldy = dense_operand(Y, "Y")
        if X.shape[1] != Y.shape[1]:
            raise ValueError("X and Y must have the same feature count")
        if out is None:
            out = torch.zeros(self.nnz, dtype=torch.float32, device=X.device)
        fn = self.lib.stile_sddmm_run_bf16 if bf16 else self.lib.stile_sddmm_run
        _lib.check(fn(self.handle, X.data_ptr(), ldx, Y.data_ptr(), ldy, out.data_ptr(), X.shape[1], _stream()),
                   "stile_sddmm_run_bf16" if bf16 else "stile_sddmm_run")
        return out

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.stile_sddmm_plan_free(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CsrMatrix:
    """A CSR matrix resident on the device for the plain CSR-row kernel."""

    def __init__(self, A, device="cuda"):
        import scipy.sparse as sp
        A = sp.csr_matrix(A)
        A.sort_indices()
        self.shape = A.shape
        self.nnz = A.nnz
        self.indptr = torch.as_tensor(A.indptr.astype(np.int32), device=device)
        self.indices = torch.as_tensor(A.indices.astype(np.int32), device=device)
        self.vals = torch.as_tensor(A.data.astype(np.float32), device=device)
        self.lib = _lib.load()
        # first row of every nonzero-balanced group of the CSR kernel
        gn = int(self.lib.stile_csr_group_nnz())
        starts = np.arange(0, max(A.nnz, 1), gn, dtype=np.int64)
        rows = np.searchsorted(A.indptr, starts, side="right") - 1
        self.group_rows = torch.as_tensor(np.minimum(rows, max(A.shape[0] - 1, 0)).astype(np.int32), device=device)

    def set_values(self, vals: torch.Tensor):
        """New values in CSR order (one per nonzero)."""
        if vals.numel() != self.nnz:
            raise ValueError("vals must have one entry per nonzero")
        self.vals.copy_(vals.detach().reshape(-1).float())

    def spmm(self, B: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        B, ldb = dense_operand(B, "B")
        N = B.shape[1]
        out, ldc, target = output_operand(out, self.shape[0], N, B.device)
        _lib.check(self.lib.stile_csr_spmm_run(self.shape[0], self.nnz, self.indptr.data_ptr(), self.indices.data_ptr(),
                                               self.vals.data_ptr(), self.group_rows.data_ptr(), B.data_ptr(), ldb,
                                               out.data_ptr(), ldc, N, _stream()), "stile_csr_spmm_run")
        return finish_output(out, target)


def plain_sddmm_plan(A) -> DeviceSddmmPlan:
    """The entry-list SDDMM over every nonzero of A (CSR order): out[t] =
    <X[row t], Y[col t]>, the plain comparator of the hybrid plans."""
    import scipy.sparse as sp
    from . import device as D
    A = sp.csr_matrix(A)
    A.sort_indices()
    dev = D.SddmmDevice(M=A.shape[0], K=A.shape[1], nnz=A.nnz,
                        mid_idx=np.repeat(np.arange(A.shape[0]), np.diff(A.indptr)).astype(np.int32),
                        j_idx=A.indices.astype(np.int32), remap=np.arange(A.nnz, dtype=np.int32),
                        bm=16, bn=16, blk_i=np.zeros(0, np.int32), blk_j=np.zeros(0, np.int32),
                        blk_indptr=np.zeros(1, np.int32), blk_dense_pos=np.zeros(0, np.int32),
                        blk_out=np.zeros(0, np.int32))
    return DeviceSddmmPlan(dev)


def launch_count() -> int:
    return int(_lib.load().stile_launch_count())
