"""Device layout of a plan: derives the arrays the sm_103a kernels read from
the reference-layout arrays produced by ``emit`` (whose index content is
left unchanged) and from the real matrix values.

SpMM (``build_spmm_device``):
  * tensor-core items -- one per (TC format, compressed 16-row block); each
    16-column slice of a block is a k-step with 16 column ids and a 16x16
    value image in the tcgen05 B-operand layout (K-major, no swizzle:
    element (n, k) at byte (n/8)*256 + (k/8)*128 + (n%8)*16 + (k%8)*2);
  * ELL items -- one per row-bucket tile, the reference's
    ``indices_k`` / ``indices_reordered_i`` arrays plus the live slot count of
    every row;
  * output rows that must not be written become -1: the sentinel row M of
    withdrawn ELL rows, rows of the padded feature space beyond M, and the
    padding rows of a partially filled tile (the reference fills them with a
    repeat of the tile's last row, which would store zeros over an owned
    row);
  * ``zero_rows``: rows without an owned (non-atomic) writer.

Values come from the real matrix, looked up by (original row, original
column) for every live entry; the reference plans on the 0/1 pattern.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from .emit import emit_sddmm_reference, emit_spmm_reference
from .plan import ELL, ONE_D, TC, TC_SDDMM

TC_BF16, TC_F16, TC_FP8, TC_SPLIT_BF16 = 1, 2, 3, 4
E4M3_MAX = 448.0


class ValueIndex:
    """(row, col) -> position in a sorted CSR matrix."""

    def __init__(self, A):
        A = sp.csr_matrix(A)
        A.sort_indices()
        self.A = A
        self.K = A.shape[1]
        rows = np.repeat(np.arange(A.shape[0], dtype=np.int64), np.diff(A.indptr))
        self.keys = rows * self.K + A.indices.astype(np.int64)

    def lookup(self, rows, cols):
        """Returns (nnz position or -1, value or 0)."""
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        q = rows * self.K + cols
        pos = np.searchsorted(self.keys, q)
        pos_c = np.minimum(pos, len(self.keys) - 1) if len(self.keys) else pos
        hit = (len(self.keys) > 0) & (pos < len(self.keys))
        if len(self.keys):
            hit = hit & (self.keys[pos_c] == q)
        ids = np.where(hit, pos_c, -1)
        vals = np.where(hit, self.A.data[pos_c] if len(self.keys) else 0.0, 0.0)
        return ids.astype(np.int64), vals


def _to_bf16_bits(x):
    """Round-to-nearest-even float32 -> bfloat16 bit patterns."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16).astype(np.uint16)
    nan = np.isnan(x)
    r[nan] = 0x7FC0
    return r


def _bf16_bits_to_f32(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def _to_f16_bits(x):
    return np.asarray(x, dtype=np.float32).astype(np.float16).view(np.uint16)


def operand_image_16bit(vals16):
    """[n_ksteps, 16 (n), 16 (k)] uint16 -> [n_ksteps, 256] in the K-major,
    no-swizzle tcgen05 operand layout (core matrices of 8 rows x 8 elements;
    element (n, k) at 16-bit index (n//8)*128 + (k//8)*64 + (n%8)*8 + k%8)."""
    nk = vals16.shape[0]
    v = vals16.reshape(nk, 2, 8, 2, 8)            # (ks, n_grp, n_in, k_grp, k_in)
    v = v.transpose(0, 1, 3, 2, 4)                # (ks, n_grp, k_grp, n_in, k_in)
    return np.ascontiguousarray(v.reshape(nk, 256))


def to_e4m3(x):
    """float32 -> (e4m3 bytes, the e4m3 values as float32): round to nearest
    even, saturated to +-448."""
    import torch
    t = torch.as_tensor(np.ascontiguousarray(x, np.float32)).clamp(-E4M3_MAX, E4M3_MAX).to(torch.float8_e4m3fn)
    return t.view(torch.uint8).numpy(), t.to(torch.float32).numpy()


def operand_image_e4m3(bytes16):
    """[n_ksteps, 16 (n), 16 (k)] e4m3 bytes -> [n_ksteps, 512] K-major,
    no-swizzle image of a K = 32 operand whose upper 16 k are zero: core
    matrices of 8 rows x 16 bytes, element (n, k) at byte (n//8)*256 +
    (k//16)*128 + (n%8)*16 + k%16."""
    nk = bytes16.shape[0]
    img = np.zeros((nk, 2, 2, 8, 16), dtype=np.uint8)     # (ks, n_grp, k_half, n_in, k_in)
    img[:, :, 0] = bytes16.reshape(nk, 2, 8, 16)
    return np.ascontiguousarray(img.reshape(nk, 512))


def fp8_row_scales(vals_f, kbeg):
    """Per (tensor-core item, row) scale: the largest |value| of the row over
    the item's k-steps / 448 (1 for an empty row).  [n_items * 16] float32."""
    n_items = len(kbeg) - 1
    out = np.ones((n_items, 16), dtype=np.float32)
    if n_items == 0 or len(vals_f) == 0:
        return out.reshape(-1)
    rowmax = np.abs(vals_f).max(axis=2)                  # [n_ks, 16]
    starts = np.asarray(kbeg[:-1], dtype=np.int64)
    nonempty = np.diff(kbeg) > 0
    red = np.maximum.reduceat(rowmax, np.minimum(starts, len(rowmax) - 1), axis=0)
    red[~nonempty] = 0.0
    s = red / E4M3_MAX
    out = np.where(s > 0, s, 1.0).astype(np.float32)
    return out.reshape(-1)


@dataclass
class SpmmDevice:
    M: int
    K: int
    nnz: int
    tc_mode: int
    tc_item_kbeg: np.ndarray
    tc_item_flags: np.ndarray
    tc_out_rows: np.ndarray
    tc_cols: np.ndarray
    tc_vals: np.ndarray        # uint8 bytes
    tc_kstep_bytes: int
    tc_nnz_id: np.ndarray
    tc_values_f32: np.ndarray  # [n_ksteps, 16, 16] exact values (for checks)
    ell_item_row0: np.ndarray
    ell_item_K: np.ndarray
    ell_item_slot0: np.ndarray
    ell_item_flags: np.ndarray
    ell_out_row: np.ndarray
    ell_row_len: np.ndarray
    ell_vals: np.ndarray
    ell_kidx: np.ndarray
    ell_nnz_id: np.ndarray
    zero_rows: np.ndarray
    # fp8 tensor tiles: scale of every (item, row) (empty otherwise)
    tc_row_scale: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))

    def stats(self):
        return {"tc_items": int(len(self.tc_item_flags)), "tc_ksteps": int(len(self.tc_cols) // 16),
                "ell_items": int(len(self.ell_item_K)), "ell_rows": int(len(self.ell_out_row)),
                "ell_slots": int(len(self.ell_kidx)), "zero_rows": int(len(self.zero_rows))}


def build_spmm_device(tiles, A, N=32, tc_mode=TC_BF16, emitted=None):
    """Device arrays for the fused SpMM of ``tiles`` over the real matrix A
    (scipy CSR, shape (M, K) of the plan, real values)."""
    A = sp.csr_matrix(A)
    A.sort_indices()
    M, K = A.shape
    vidx = ValueIndex(A)
    if emitted is None:
        emitted = emit_spmm_reference(tiles, M, N)
    formats, args, _ = emitted

    # ---------------- tensor-core items ----------------
    kbeg_parts, flags, out_rows = [np.zeros(1, np.int64)], [], []
    cols_l, vals_l, live_l, srcr_l = [], [], [], []
    n_ks = 0
    for f, arr in zip(formats, args):
        if f.template != TC:
            continue
        a, i_idx, indptr, indices = arr
        tsz = int(f.tile_sizes[0][1])
        nnzb, _, kw = a.shape
        if indices.ndim == 1:
            # column-ordered blocks (TC_k_notsorted): a k-block position per
            # block; columns past K carry zero values and read row K - 1
            indices = np.minimum(indices.astype(np.int64)[:, None] * kw + np.arange(kw)[None, :], K - 1)
        assert tsz == 16 and kw % 16 == 0, "tensor-core blocks are 16 rows x 16k columns"
        nsub = kw // 16
        tiles_sorted = sorted(f.tiles, key=lambda t: tuple(t.tile_pos))
        atomic = bool(f.params["real_atomic"])
        mb = len(indptr) - 1
        # rows of every block (from its tile's row range), -1 past the end
        src = np.full((nnzb, 16), -1, dtype=np.int64)
        n_real_blk = np.zeros(nnzb, dtype=np.int64)
        for j, t in enumerate(tiles_sorted):
            r0, r1 = t.tile_i_rng
            src[j, :r1 - r0 + 1] = t.op.i_perm[r0:r1 + 1]
            n_real_blk[j] = r1 - r0 + 1
        firsts = indptr[:-1].astype(np.int64)
        if i_idx.ndim == 2:
            rows = i_idx.astype(np.int64).copy()
        else:
            rows = i_idx.astype(np.int64)[:, None] * 16 + np.arange(16, dtype=np.int64)[None, :]
        rows[np.arange(16)[None, :] >= n_real_blk[firsts][:, None]] = -1
        rows[rows >= M] = -1
        out_rows.append(rows)
        flags.append(np.full(mb, 1 if atomic else 0, dtype=np.int64))
        steps_per_item = np.diff(indptr).astype(np.int64) * nsub
        kbeg_parts.append(n_ks + np.cumsum(steps_per_item))
        n_ks += int(nnzb * nsub)
        cols_l.append(indices.reshape(nnzb * nsub, 16).astype(np.int64))
        v = a.reshape(nnzb, 16, nsub, 16).transpose(0, 2, 1, 3).reshape(nnzb * nsub, 16, 16)
        lv = v != 0
        lv &= (np.arange(16)[None, :] < np.repeat(n_real_blk, nsub)[:, None])[:, :, None]
        live_l.append(lv)
        srcr_l.append(np.repeat(src, nsub, axis=0))
    kbeg = np.concatenate(kbeg_parts)
    if n_ks:
        cols = np.concatenate(cols_l)
        live = np.concatenate(live_l)
        srcr = np.concatenate(srcr_l)
        R = np.broadcast_to(srcr[:, :, None], (n_ks, 16, 16))
        Cc = np.broadcast_to(cols[:, None, :], (n_ks, 16, 16))
        ids, v = vidx.lookup(np.where(live, R, 0).reshape(-1), np.where(live, Cc, 0).reshape(-1))
        ids = ids.reshape(n_ks, 16, 16)
        v = v.reshape(n_ks, 16, 16)
        if np.any(live & (ids < 0)):
            raise ValueError("plan covers an entry that is not a nonzero of A")
        nnz_ids = np.where(live, ids, -1).reshape(n_ks, 256).astype(np.int32)
        vals_f = np.where(live, v, 0.0).astype(np.float32)
        cols = cols.astype(np.int32)
    else:
        cols = np.zeros((0, 16), np.int32)
        vals_f = np.zeros((0, 16, 16), np.float32)
        nnz_ids = np.zeros((0, 256), np.int32)
    flags = np.concatenate(flags) if flags else np.zeros(0, np.int64)
    if tc_mode == TC_BF16:
        img = operand_image_16bit(_to_bf16_bits(vals_f).reshape(n_ks, 16, 16))
        tc_bytes = 512
    elif tc_mode == TC_F16:
        img = operand_image_16bit(_to_f16_bits(vals_f).reshape(n_ks, 16, 16))
        tc_bytes = 512
    elif tc_mode == TC_SPLIT_BF16:
        hi = _to_bf16_bits(vals_f)
        lo = _to_bf16_bits(vals_f - _bf16_bits_to_f32(hi))
        img = np.concatenate([operand_image_16bit(hi.reshape(n_ks, 16, 16)),
                              operand_image_16bit(lo.reshape(n_ks, 16, 16))], axis=1)
        tc_bytes = 1024
    elif tc_mode == TC_FP8:
        row_scale = fp8_row_scales(vals_f, np.asarray(kbeg, dtype=np.int64))
        item_of = np.repeat(np.arange(len(kbeg) - 1), np.diff(np.asarray(kbeg, dtype=np.int64)))
        s = row_scale.reshape(-1, 16)[item_of] if n_ks else np.ones((0, 16), np.float32)
        b8, _ = to_e4m3(vals_f / s[:, :, None] if n_ks else vals_f)
        img = operand_image_e4m3(b8.reshape(n_ks, 16, 16))
        tc_bytes = 512
    else:
        raise ValueError(f"unsupported tensor-tile mode {tc_mode}")
    tc_vals = np.ascontiguousarray(img).view(np.uint8).reshape(-1)

    # ---------------- ELL items ----------------
    row0 = [0]
    eK, eslot, eflags, eout, elen, evals, ekidx, enid = [], [], [], [], [], [], [], []
    n_rows = 0
    n_slots = 0
    for f, arr in zip(formats, args):
        if f.template != ELL:
            continue
        _, kidx, iout = arr
        I = int(np.prod([int(x) for x in f.tile_sizes[0][1:]]))
        Kl = kidx.shape[1]
        atomic = bool(f.params["real_atomic"])
        nt = len(f.tiles)
        # every tile of the format at once: rows c * I .. (c + 1) * I - 1
        # belong to tile c, whose first n_real rows are real
        lens = np.zeros(nt * I, dtype=np.int64)
        n_real = np.empty(nt, dtype=np.int64)
        for c, t in enumerate(f.tiles):
            cov = t.covered
            n_real[c] = cov.shape[0]
            lens[c * I:c * I + n_real[c]] = np.diff(sp.csr_matrix(cov).indptr)
        orow = iout[:nt * I].astype(np.int64).copy()
        orow[np.arange(nt * I) % I >= np.repeat(n_real, I)] = -1
        orow[orow >= M] = -1
        if not atomic:
            orow[lens == 0] = -1
        ki = kidx[:nt * I].astype(np.int64)
        live = np.arange(Kl)[None, :] < lens[:, None]
        live &= (orow >= 0)[:, None]
        R = np.repeat(np.maximum(orow, 0)[:, None], Kl, axis=1)
        ids, v = vidx.lookup(np.where(live, R, 0), np.where(live, ki, 0))
        ids = np.where(live, ids, -1)
        v = np.where(live, v, 0.0)
        if np.any(live & (ids < 0)):
            raise ValueError("plan covers an entry that is not a nonzero of A")
        eK.extend([Kl] * nt)
        eslot.extend((n_slots + I * Kl * np.arange(nt)).tolist())
        eflags.extend([1 if atomic else 0] * nt)
        eout.append(orow)
        elen.append(np.where(orow >= 0, lens, 0))
        evals.append(v.reshape(-1))
        ekidx.append(ki.reshape(-1))
        enid.append(ids.reshape(-1))
        row0.extend((n_rows + I * (np.arange(nt) + 1)).tolist())
        n_rows += I * nt
        n_slots += I * Kl * nt

    def cat(xs, dt):
        return np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)

    ell_out = cat(eout, np.int32)
    tc_rows = np.concatenate(out_rows).reshape(-1).astype(np.int32) if out_rows else np.zeros(0, np.int32)
    tc_flags = np.asarray(flags, dtype=np.int32)
    ell_flags = np.asarray(eflags, dtype=np.int32)
    # owned rows: stored by exactly one non-atomic writer
    owned = []
    if len(tc_rows):
        rr = tc_rows.reshape(-1, 16)
        owned.append(rr[tc_flags == 0].reshape(-1))
    if len(ell_out):
        per_row_flag = np.repeat(ell_flags, np.diff(np.asarray(row0)))
        owned.append(ell_out[per_row_flag == 0])
    owned = np.concatenate(owned) if owned else np.zeros(0, np.int32)
    owned = owned[owned >= 0]
    uniq, cnt = np.unique(owned, return_counts=True)
    if np.any(cnt > 1):
        raise ValueError(f"owned output rows with more than one writer: {uniq[cnt > 1][:10]}")
    zero_rows = np.setdiff1d(np.arange(M, dtype=np.int32), uniq.astype(np.int32)).astype(np.int32)

    return SpmmDevice(
        M=M, K=K, nnz=int(A.nnz), tc_mode=tc_mode,
        tc_item_kbeg=np.asarray(kbeg, dtype=np.int32), tc_item_flags=tc_flags,
        tc_out_rows=tc_rows, tc_cols=cols.reshape(-1).astype(np.int32), tc_vals=tc_vals,
        tc_kstep_bytes=tc_bytes, tc_nnz_id=nnz_ids.reshape(-1).astype(np.int32), tc_values_f32=vals_f,
        ell_item_row0=np.asarray(row0, dtype=np.int32), ell_item_K=np.asarray(eK, dtype=np.int32),
        ell_item_slot0=np.asarray(eslot, dtype=np.int32), ell_item_flags=ell_flags,
        ell_out_row=ell_out, ell_row_len=cat(elen, np.int32), ell_vals=cat(evals, np.float32),
        ell_kidx=cat(ekidx, np.int32), ell_nnz_id=cat(enid, np.int32), zero_rows=zero_rows,
        tc_row_scale=row_scale if tc_mode == TC_FP8 else np.zeros(0, np.float32))


@dataclass
class SddmmDevice:
    M: int
    K: int
    nnz: int
    mid_idx: np.ndarray
    j_idx: np.ndarray
    remap: np.ndarray
    bm: int
    bn: int
    blk_i: np.ndarray
    blk_j: np.ndarray
    blk_indptr: np.ndarray
    blk_dense_pos: np.ndarray
    blk_out: np.ndarray


def build_sddmm_device(tiles, shape, nnz, emitted=None):
    if emitted is None:
        emitted = emit_sddmm_reference(tiles)
    formats, args = emitted
    mids, js, rms = [], [], []
    bi, bj, dps, outs, counts = [], [], [], [], []
    bm = bn = 16
    for f, arr in zip(formats, args):
        if f.template == ONE_D:
            mid, jj, rm, _ = arr
            mids.append(mid); js.append(jj); rms.append(rm)
        elif f.template == TC_SDDMM:
            i_idx, j_idx, indptr, dpos, ids, _ = arr
            bm, bn = i_idx.shape[1], j_idx.shape[1]
            bi.append(i_idx.reshape(-1)); bj.append(j_idx.reshape(-1))
            dps.append(dpos); outs.append(ids); counts.append(np.diff(indptr))

    def cat(xs):
        return np.concatenate(xs).astype(np.int32) if xs else np.zeros(0, np.int32)

    cnt = np.concatenate(counts) if counts else np.zeros(0, np.int64)
    indptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    return SddmmDevice(M=shape[0], K=shape[1], nnz=int(nnz), mid_idx=cat(mids), j_idx=cat(js),
                       remap=cat(rms), bm=int(bm), bn=int(bn), blk_i=cat(bi), blk_j=cat(bj),
                       blk_indptr=indptr, blk_dense_pos=cat(dps), blk_out=cat(outs))
