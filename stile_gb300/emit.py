"""Tile-format emitter: packs a selected plan into device arrays.

Two layers:

1. ``emit_spmm_reference`` / ``emit_sddmm_reference`` produce, per format,
   the arrays the reference's packer produces for the same plan
   (``prepare_inputs_BSPMM``, my_fuse_formats.py:3321-3537;
   ``prepare_inputs_BSDDMM``, :3544-3678) -- same shapes, same index
   content, same padding fill values.  Values are the covered-entry values
   of the plan (the reference plans on a 0/1 pattern, so they are 1.0).

2. ``build_spmm_device`` / ``build_sddmm_device`` derive the arrays the
   sm_103a kernels consume from (1): the real matrix values looked up by
   (original row, original column), TC block values converted to the tensor
   core operand type and permuted into the shared-memory image of one
   ``tcgen05.mma`` K-step, sentinel output rows (-1) for rows that must not
   be written, and the list of output rows that no owned (non-atomic) tile
   stores, which the callee zeroes before the fused kernel runs.
   The index arrays themselves are not changed.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

from .plan import ELL, ONE_D, TC, TC_SDDMM, Format, group_formats, tile_extent


# ---------------------------------------------------------------------------
# output shape (set_params_BSPMM, my_fuse_formats.py:2670-2830)
# ---------------------------------------------------------------------------
def padded_j_tc(n, mma_n=16):
    """``get_padded_j_TC``: feature count padded for TC formats."""
    if n < mma_n:
        return mma_n
    if n > mma_n:
        return int(math.ceil(n / (2 * mma_n)) * 2 * mma_n)
    return n


def spmm_out_shape(formats, M, N):
    max_i, max_j = M + 1, N
    for f in formats:
        if f.template == TC:
            ts = int(f.tile_sizes[0][1])
            max_i = max(max_i, int(math.ceil(M / ts) * ts))
            max_j = max(max_j, padded_j_tc(N, 16))
    return max_i, max_j


# ---------------------------------------------------------------------------
# reference-layout emission
# ---------------------------------------------------------------------------
def _csr(cov):
    return cov if sp.isspmatrix_csr(cov) else sp.csr_matrix(cov)


def _emit_ell(fmt):
    tiles = fmt.tiles
    ilen, klen = tile_extent(fmt.tile_sizes[0]), tile_extent(fmt.tile_sizes[2])
    nt = len(tiles)
    a = np.zeros((ilen * nt, klen))
    indices_k = np.empty((ilen * nt, klen), dtype=np.int64)
    i_out = np.empty(ilen * nt, dtype=np.int64)
    for c, t in enumerate(tiles):
        op = t.op
        base = c * ilen
        indices_k[base:base + ilen] = op.k_perm[0]
        if t.tile_i_rng is None:
            i_out[base:base + ilen] = t.i_vals[-1]
        else:
            i_out[base:base + ilen] = op.i_perm[op.hyb_new_rows[-1]]
        cov = _csr(t.covered)
        nnz_r = np.diff(cov.indptr)
        rows = np.repeat(np.arange(cov.shape[0]), nnz_r)
        slot = np.arange(cov.nnz) - np.repeat(cov.indptr[:-1], nnz_r)
        a[base + rows, slot] = cov.data
        indices_k[base + rows, slot] = op.k_perm[cov.indices]
        n_rows = cov.shape[0]
        if t.tile_i_rng is None:
            i_out[base:base + n_rows] = t.i_vals
        else:
            r0, r1 = t.tile_i_rng
            i_out[base:base + n_rows] = op.i_perm[op.hyb_new_rows[r0:r1 + 1]]
    a = a.reshape(nt, ilen * klen)
    return a, indices_k.astype(np.int32), i_out.astype(np.int32)


def _sorted_tc_tiles(tiles):
    return sorted(tiles, key=lambda t: tuple(t.tile_pos))


def _emit_tc(fmt):
    tiles = _sorted_tc_tiles(fmt.tiles)
    ilen, klen = tile_extent(fmt.tile_sizes[0]), tile_extent(fmt.tile_sizes[2])
    nt = len(tiles)
    a = np.zeros((nt, ilen, klen))
    for c, t in enumerate(tiles):
        cov = _csr(t.covered)
        rows = np.repeat(np.arange(cov.shape[0]), np.diff(cov.indptr))
        np.add.at(a[c], (rows, cov.indices), cov.data)
    poi_is, counts = np.unique([int(t.tile_pos[0]) for t in tiles], return_counts=True)
    indptr = np.concatenate(([0], np.cumsum(counts)))
    indices = np.empty((nt, klen), dtype=np.int64)
    for c, t in enumerate(tiles):
        op = t.op
        order = op.blk_k_vals[int(t.tile_pos[0])]
        indices[c, :] = op.k_perm[order[t.k_vals[-1]]]
        ncol = _csr(t.covered).shape[1]
        indices[c, :ncol] = op.k_perm[order[t.k_vals]]
    p = fmt.params
    if p["idx_reordered"][0] or p["real_atomic"]:
        i_indices = np.empty((len(poi_is), ilen), dtype=np.int64)
        for c, ti in enumerate(indptr[:-1]):
            t = tiles[ti]
            op = t.op
            r0, r1 = t.tile_i_rng
            i_indices[c, :] = op.i_perm[r1]
            nrow = _csr(t.covered).shape[0]
            i_indices[c, :nrow] = op.i_perm[r0:r1 + 1]
    else:
        i_indices = poi_is
    if tiles[0].op.TC_k_notsorted:
        indices = np.asarray([int(t.tile_pos[2]) for t in tiles])
    return (a, np.asarray(i_indices).astype(np.int32), indptr.astype(np.int32),
            indices.astype(np.int32))


def emit_spmm_reference(tiles, M, N, formats=None):
    """Returns (formats, per-format arg tuples, out_shape)."""
    if formats is None:
        formats = group_formats(tiles)
    out = []
    for f in formats:
        if f.template == ELL:
            out.append(_emit_ell(f))
        elif f.template == TC:
            out.append(_emit_tc(f))
        else:
            raise ValueError(f"not an SpMM template: {f.template}")
    return formats, out, spmm_out_shape(formats, M, N)


def _emit_1d(fmt):
    tiles = fmt.tiles
    ts = int(fmt.tile_sizes[0])
    mid, jj, rm = [], [], []
    for t in tiles:
        op = t.op
        s = slice(int(t.tile_pos[0]) * ts, (int(t.tile_pos[0]) + 1) * ts)
        mid.append(op.ori_row_ids_1d[s])
        jj.append(op.ori_col_ids_1d[s])
        rm.append(op.nnz_id_1d[s])
    mid, jj, rm = np.concatenate(mid), np.concatenate(jj), np.concatenate(rm)
    real = int(fmt.params["ty"]) * int(fmt.params["group_size"])
    to_pad = int(math.ceil(len(mid) / real) * real - len(mid))
    mid = np.concatenate([mid, np.full(to_pad, mid[-1])])
    jj = np.concatenate([jj, np.full(to_pad, jj[-1])])
    rm = np.concatenate([rm, np.full(to_pad, rm[-1])])
    return mid.astype(np.int32), jj.astype(np.int32), rm.astype(np.int32), np.zeros(len(rm))


def _emit_tc_sddmm(fmt):
    tiles = fmt.tiles
    ts_i, ts_k = int(fmt.tile_sizes[0][1]), int(fmt.tile_sizes[2][1])
    op = tiles[0].op
    # a block cut short by the matrix edge (the reference pads its shapes to
    # full blocks, so it never has one) repeats its last row / column, as
    # the SpMM packer pads its column indices; only live entries are computed
    i_indices = np.empty((len(tiles), ts_i), dtype=np.int64)
    j_indices = np.empty((len(tiles), ts_k), dtype=np.int64)
    for c, t in enumerate(tiles):
        rows = op.i_perm[t.tile_i_rng[0]:t.tile_i_rng[1] + 1]
        cols = op.k_perm[op.blk_k_vals[int(t.tile_pos[0])][t.tile_k_rng[0]:t.tile_k_rng[1] + 1]]
        i_indices[c, :len(rows)], i_indices[c, len(rows):] = rows, rows[-1]
        j_indices[c, :len(cols)], j_indices[c, len(cols):] = cols, cols[-1]
    cache = {}
    dense_pos, ids, counts = [], [], []
    for t in tiles:
        r = int(t.tile_pos[0])
        if r not in cache:
            cache[r] = op.nnz_id_matrix[r * ts_i:(r + 1) * ts_i, :]
        # selecting the tile's columns of the block's order is the
        # reference's "permute every column, then slice the range"
        csc = cache[r][:, op.blk_k_vals[r][t.tile_k_rng[0]:t.tile_k_rng[1] + 1]].tocsc()
        dense_pos.append(np.repeat(np.arange(csc.shape[1]), csc.getnnz(axis=0)) + csc.indices * ts_k)
        ids.append(csc.data - 1)
        counts.append(csc.nnz)
    indptr = np.cumsum([0] + counts)
    c = np.zeros((len(tiles), ts_i, ts_k))
    return (i_indices.astype(np.int32), j_indices.astype(np.int32), indptr.astype(np.int32),
            np.concatenate(dense_pos).astype(np.int32), np.concatenate(ids).astype(np.int32), c)


def emit_sddmm_reference(tiles, formats=None):
    if formats is None:
        formats = group_formats(tiles)
    out = []
    for f in formats:
        if f.template == ONE_D:
            out.append(_emit_1d(f))
        elif f.template == TC_SDDMM:
            out.append(_emit_tc_sddmm(f))
        else:
            raise ValueError(f"not an SDDMM template: {f.template}")
    return formats, out
