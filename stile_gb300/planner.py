"""Format search: tile generation, greedy selection with local search and
withdraw over a cost model -- the reference's planner, restated.

Reference flow (MY_sparse/): ``gen_candidate_formats`` (gen_formats_v2.py
:1510-1835, :1837-1900) builds one ELL operator (rows stably sorted by
decreasing length and folded at the bucket size) and one tensor-core
operator (the densest of original / length-sorted row orders, columns of
every 16-row block stably sorted by decreasing count);
``greedy_search_use_cost_model_lower_bound`` (my_search_formats.py:263-833)
first picks tensor-core tiles block row by block row
(``search_TC_tiles_only_by_rows``, my_branch_and_bound.py:238-389), then
repeatedly takes the tile with the lowest predicted cost per newly covered
element, widened by a local search to every tile within
``1 + max_avg_cost_diff`` of it (:1117-1647), regenerating next-level ELL
operators from the uncovered elements after every tensor-core pick
(:1051-1094); ``post_process_for_withdraw`` (:1652-1759) finally drops tiles
replaced by whole-row tensor-core tiles.

Implementation: every operator is a permuted view of the matrix's nonzeros
and carries, per entry, the nonzero id; covering is one boolean mask over
the ids, so "position space updates" are mask lookups and all per-tile
counts are vectorised prefix sums / bincounts.  The k order of a
tensor-core block is stored as its non-empty columns only (the empty tail of
the reference's full-length order is ascending and computed on demand).
"""
from __future__ import annotations

import math
import warnings
from fractions import Fraction

import numpy as np
import scipy.sparse as sp

from .cost_model import A100_FP16, CostModel
from .plan import ELL, ONE_D, TC, TC_SDDMM, OpSpace, Plan, Tile

TC_PARAMS = {"mma_shape_str": "m16n16k16"}
ONE_D_PARAMS = {"tx": 8, "ty": 4, "vec_size": 4, "group_size": 8, "max_bucket_size": 32}


# ---------------------------------------------------------------------------
# pattern
# ---------------------------------------------------------------------------
class Pattern:
    """The 0/1 pattern of A with nonzero ids 0..nnz-1 in CSR order."""

    def __init__(self, A):
        A = sp.csr_matrix(A)
        A.sum_duplicates()
        A.sort_indices()
        self.M, self.K = A.shape
        self.indptr = A.indptr.astype(np.int64)
        self.indices = A.indices.astype(np.int64)
        self.nnz = int(A.nnz)
        self.row_nnz = np.diff(self.indptr)
        self.row_of = np.repeat(np.arange(self.M, dtype=np.int64), self.row_nnz)

    def sub_row_nnz(self, ids):
        return np.bincount(self.row_of[ids], minlength=self.M)


def _run_counts(code):
    """(values, counts) of a nondecreasing integer array: np.unique's result
    without its sort."""
    if len(code) == 0:
        return code, np.zeros(0, dtype=np.int64)
    starts = np.flatnonzero(np.concatenate([[True], code[1:] != code[:-1]]))
    return code[starts], np.diff(np.append(starts, len(code)))


def _tile_csr(rows, cols, shape):
    """The 0/1 CSR of a tile's covered entries (unique (row, column) pairs),
    canonical as scipy's COO -> CSR conversion makes it (rows, then columns
    ascending), built directly."""
    R, C = shape
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    o = np.argsort(rows * C + cols)
    indptr = np.zeros(R + 1, dtype=np.int32)
    np.cumsum(np.bincount(rows, minlength=R), out=indptr[1:])
    return sp.csr_matrix((np.ones(len(rows)), cols[o].astype(np.int32), indptr), shape=shape)


def estimate_max_bucket_size(nnz, sm_num=108):
    """Bucket (fold) length of ELL rows from the expected occupancy
    (my_search_formats.py:965-981; 256-thread blocks, 2048 threads / SM)."""
    blk_per_sm = 2048 / 256
    cands = [8 * (2 ** i) for i in range(2, 6)][::-1]
    for cand in cands:
        if nnz / (cand / 2) / sm_num >= 0.5 * blk_per_sm:
            return cand // 8
    return cands[-1] // 8


def tc_tile_sizes(op_type="spmm", k_notsorted=False):
    """get_TC_tile_sizes (gen_formats_v2.py:1237-1283): with the columns kept
    in order (TC_k_notsorted) only 16x32x16 tiles, for both operators."""
    if k_notsorted:
        return [((None, 16), (None, 32), (None, 16))]
    if op_type == "sddmm":
        return [((None, 16), (None, 16 * (2 ** j)), (None, 16)) for j in range(3)]
    return [((None, 16), (None, 32), (None, 16 * i)) for i in range(10, 0, -1)]


# ---------------------------------------------------------------------------
# ELL operator
# ---------------------------------------------------------------------------
class EllOp:
    """Rows of the covered-entry subset ``ids`` stably sorted by decreasing
    length and folded into rows of at most ``mbs`` entries
    (reorder_idx :820-851, pad_irregular_idx :1065-1121)."""

    def __init__(self, pat: Pattern, ids, mbs, op_id):
        self.pat = pat
        self.op_id = op_id
        self.mbs = mbs
        ids = np.asarray(ids, dtype=np.int64)   # CSR order of the subset
        if len(ids) > 1 and not np.all(ids[1:] > ids[:-1]):
            ids = np.sort(ids)
        rn = pat.sub_row_nnz(ids)
        self.row_nnz_pos = None
        self.i_perm = np.argsort(-rn, kind="stable")
        rn_sorted = rn[self.i_perm]
        self.new_row_nums = np.maximum(np.ceil(rn_sorted / mbs), 1).astype(np.int64)
        self.hyb_new_rows = np.repeat(np.arange(pat.M, dtype=np.int64), self.new_row_nums)
        self.hyb_ori_row_ends = np.cumsum(self.new_row_nums) - 1
        sb = int(np.searchsorted(-rn_sorted, -mbs))
        self.short_begin = len(self.hyb_new_rows) if sb == len(rn_sorted) else int(self.hyb_ori_row_ends[sb])
        self.n_folded = len(self.hyb_new_rows)
        # entries in position order: rows in i_perm order, each row's entries
        # in column order, chunks of mbs -> folded rows.  ``ids`` is in CSR
        # order (rows ascending, columns ascending within a row), so the
        # order is the subset's row segments taken in i_perm order.
        sub_start = np.concatenate([[0], np.cumsum(rn)[:-1]])
        out_start = np.concatenate([[0], np.cumsum(rn_sorted)[:-1]])
        order = np.repeat(sub_start[self.i_perm] - out_start, rn_sorted) + np.arange(len(ids), dtype=np.int64)
        self.ids = ids[order]
        self.cols = pat.indices[self.ids]
        # entries per folded row: mbs for every fold of a row but its last,
        # which holds the rest (0 for an empty row's single fold)
        fold_first = self.hyb_ori_row_ends - self.new_row_nums + 1
        j = np.arange(self.n_folded, dtype=np.int64) - fold_first[self.hyb_new_rows]
        fold_len = np.clip(rn_sorted[self.hyb_new_rows] - j * mbs, 0, mbs)
        self.indptr = np.zeros(self.n_folded + 1, dtype=np.int64)
        np.cumsum(fold_len, out=self.indptr[1:])
        # folded row of every entry
        self.frow = np.repeat(np.arange(self.n_folded, dtype=np.int64), fold_len)
        self.init_nnz = np.diff(self.indptr)
        self.getnnz_minus = -self.init_nnz[self.short_begin:]
        self._kis_cache = {}

    # uncovered entries per folded row
    def upd_rows(self, uncovered):
        live = uncovered[self.ids]
        c = np.concatenate([[0], np.cumsum(live)])
        return c[self.indptr[1:]] - c[self.indptr[:-1]], c

    def tile_shapes(self, N):
        """(I, J, K) candidates: I*K = 8*mbs, J = 32, 256 <= I*J, I*J % 128 == 0
        (tile_size_heuristics :1188-1242, get_tile_sizes_idx :1926-1980)."""
        Is = [2 ** t for t in range(int(math.log(self.n_folded, 2)) + 1)]
        Ks = [2 ** t for t in range(int(math.log(self.mbs, 2)) + 1)]
        out = []
        for I in Is:
            for K in Ks:
                if (I * 32) % 128 != 0 or I * 32 < 256 or I * K != self.mbs * 8:
                    continue
                out.append((I, 32, K))
        return out

    def valid_positions(self, I, K):
        """get_valid_tile_pos_list_for_ELL (my_branch_and_bound.py:16-53)."""
        t0 = int(np.searchsorted(self.getnnz_minus, -K)) + self.short_begin
        t1 = int(np.searchsorted(self.getnnz_minus, -(K // 2))) + self.short_begin
        list1 = list(range(math.ceil(t0 / I), (t1 - 1) // I + 1))
        if list1 and (list1[-1] + 1) * I < self.n_folded:
            list1.append(list1[-1] + 1)
        if K == self.mbs:
            list2 = list(range((self.short_begin - 1) // I + 1))
            return list2 + list1
        return list1

    def k_is(self, I, K, pos_is):
        """Distinct columns per tile in the operator's initial entries (+ the
        fill column 0 when the tile is not full)."""
        key = I
        if key not in self._kis_cache:
            n_t = math.ceil(self.n_folded / I)
            if not hasattr(self, "_cf_col"):
                # by column, then folded row: the entries are in folded-row
                # order, so a CSR -> CSC transposition of their indices is
                # that order (a counting sort, linear in the entries)
                o = sp.csr_matrix((np.arange(len(self.cols), dtype=np.int64), self.cols, self.indptr),
                                  shape=(self.n_folded, self.pat.K)).tocsc().data
                self._cf_col = self.cols[o]
                self._cf_frow = self.frow[o]
                self._cf_colchg = self._cf_col[1:] != self._cf_col[:-1]
                # highest bit in which each entry's folded row differs from
                # the previous entry's of the same column (63: first entry of
                # its column): for I = 2^t the entry opens a new (segment,
                # column) pair exactly when that bit is >= t
                fr = self._cf_frow
                lvl = np.full(len(fr), 63, dtype=np.int8)
                if len(fr) > 1:
                    x = fr[1:] ^ fr[:-1]
                    hb = (np.frexp(np.maximum(x, 1).astype(np.float64))[1] - 1).astype(np.int8)
                    lvl[1:] = np.where(self._cf_colchg, 63, hb)
                self._cf_lvl = lvl
                self._cf_zero_frow = fr[self._cf_col == 0]
            col = self._cf_col
            if I & (I - 1) == 0:
                t = I.bit_length() - 1
                first = self._cf_lvl >= t
                distinct = np.bincount(self._cf_frow[first] >> t, minlength=n_t)
                has0 = np.zeros(n_t, dtype=bool)
                has0[self._cf_zero_frow >> t] = True
            else:
                seg = self._cf_frow // I
                # entries sorted by (column, folded row): a (segment, column)
                # pair is new wherever the column or the segment changes
                first = np.ones(len(col), dtype=bool)
                if len(col) > 1:
                    first[1:] = self._cf_colchg | (seg[1:] != seg[:-1])
                distinct = np.bincount(seg[first], minlength=n_t)
                has0 = np.zeros(n_t, dtype=bool)
                has0[seg[col == 0]] = True
            self._kis_cache[key] = (distinct, has0)
        distinct, has0 = self._kis_cache[key]
        pos_is = np.asarray(pos_is, dtype=np.int64)
        s = self.indptr[np.minimum(I * pos_is, self.n_folded)]
        e = self.indptr[np.minimum(I * (pos_is + 1), self.n_folded)]
        pads = (e - s) < (I * K)
        return distinct[pos_is] + (pads & ~has0[pos_is]).astype(np.int64)

    def space(self):
        return OpSpace(op_id=self.op_id, template=ELL, i_perm=self.i_perm,
                       k_perm=np.arange(self.pat.K, dtype=np.int64),
                       idx_reordered=(True, False, False), hyb_new_rows=self.hyb_new_rows,
                       hyb_ori_row_ends=self.hyb_ori_row_ends, hyb_short_begin_row=self.short_begin)


# ---------------------------------------------------------------------------
# tensor-core operator
# ---------------------------------------------------------------------------
class TcOp:
    """16-row blocks of a row order; in each block the columns are stably
    sorted by decreasing count (condense_for_TC_tile :1004-1039), or, with
    ``k_notsorted`` (TC_k_notsorted, :1025-1031 and set_init_blk_nums
    :1328-1335), kept in column order, so that a tile at k position p is the
    16-column block [16p, 16p + 16) and only non-empty blocks are tiles.
    ``k_by_count=False`` (reorder_k_by_nnz=False, :1036-1038) puts the
    non-empty columns first in column order instead of by decreasing count."""

    def __init__(self, pat: Pattern, i_perm, op_id, op_type="spmm", ids=None, bs=16, k_notsorted=False,
                 k_by_count=True):
        self.pat = pat
        self.op_id = op_id
        self.bs = bs
        self.op_type = op_type
        self.k_notsorted = bool(k_notsorted)
        self.i_perm = np.asarray(i_perm, dtype=np.int64)
        self.reordered = not np.array_equal(self.i_perm, np.arange(pat.M))
        inv = np.empty(pat.M, dtype=np.int64)
        inv[self.i_perm] = np.arange(pat.M)
        self.inv = inv
        self.n_blk = math.ceil(pat.M / bs)
        ids = np.arange(pat.nnz, dtype=np.int64) if ids is None else np.sort(ids)
        prow = inv[pat.row_of[ids]]
        blk = prow // bs
        col = pat.indices[ids]
        # entries grouped by (block, column), each group in the order of
        # ``ids`` (a stable sort: rows are sorted runs, so it merges runs)
        code = blk * pat.K + col
        order = np.argsort(code, kind="stable")
        sc = code[order]
        starts = np.flatnonzero(np.concatenate([[True], sc[1:] != sc[:-1]])) if len(sc) else np.zeros(0, np.int64)
        ucode = sc[starts]
        cnt = np.diff(np.append(starts, len(sc)))
        ublk = ucode // pat.K
        ucol = ucode % pat.K
        if self.k_notsorted or not k_by_count:
            # by block, then column
            o = np.arange(len(ucode))
        else:
            # by block, decreasing count, column: one integer key (unique,
            # so any sort gives the order a stable lexsort would)
            cmax = int(cnt.max()) if len(cnt) else 0
            o = np.argsort((ublk * (cmax + 1) + (cmax - cnt)) * pat.K + ucol)
        ublk, ucol, cnt, starts = ublk[o], ucol[o], cnt[o], starts[o]
        self.nonempty = np.bincount(ublk, minlength=self.n_blk)
        self.kstart = np.concatenate([[0], np.cumsum(self.nonempty)])
        self.kord_cols = ucol                       # concatenated per block
        # entries by block, then position in the block's order (the groups
        # in that order); ties (one column, several rows) keep ``ids``' order
        first = np.repeat(np.cumsum(cnt) - cnt, cnt)
        eo = order[np.repeat(starts, cnt) + np.arange(len(order)) - first]
        self.ids = ids[eo]
        self.blk = blk[eo]
        if self.k_notsorted:
            self.pos = col[eo]
        else:
            self.pos = np.repeat(np.arange(len(ucode)) - self.kstart[ublk], cnt)
        self.prow = prow[eo]
        self.bptr = np.concatenate([[0], np.cumsum(np.bincount(self.blk, minlength=self.n_blk))])
        # positions a block's counts run over: its non-empty prefix, or (in
        # column order) up to its last non-empty column
        if self.k_notsorted:
            self.extent = np.zeros(self.n_blk, dtype=np.int64)
            np.maximum.at(self.extent, ublk, ucol + 1)
        else:
            self.extent = self.nonempty
        self.blk_nums = {}
        self.blk_ks = {}
        for ts in tc_tile_sizes(op_type, self.k_notsorted):
            Kt = ts[2][1]
            if self.k_notsorted:
                nch = -(-pat.K // Kt)
                ch = np.unique(ublk * nch + ucol // Kt)
                cb = ch // nch
                self.blk_nums[ts] = np.bincount(cb, minlength=self.n_blk).astype(np.int64)
                cptr = np.concatenate([[0], np.cumsum(self.blk_nums[ts])])
                self.blk_ks[ts] = (ch % nch, cptr)
            else:
                self.blk_nums[ts] = np.ceil(self.nonempty / Kt).astype(np.int64)

    def row_positions(self, ts, b):
        """k positions of the tiles that cover block b whole: the first
        blk_nums of its order, or (in column order) its non-empty column
        blocks (``blk_ks``)."""
        if self.k_notsorted:
            ks, cptr = self.blk_ks[ts]
            return [int(x) for x in ks[cptr[b]:cptr[b + 1]]]
        return list(range(int(self.blk_nums[ts][b])))

    def density(self):
        """select_the_densest_tensor_for_TC_tiles (:1286-1309): nnz over
        16x16 blocks touched."""
        tot = int(np.sum(np.ceil(self.nonempty / 16))) * 256
        return self.pat.nnz / tot if tot else 0.0

    def kvals(self, b, positions):
        """Columns at ``positions`` of block b's order (non-empty columns, then
        the remaining columns ascending)."""
        positions = np.asarray(positions, dtype=np.int64)
        if self.k_notsorted:
            return positions.copy()
        ne = int(self.nonempty[b])
        head = self.kord_cols[self.kstart[b]:self.kstart[b + 1]]
        out = np.empty(positions.shape, dtype=np.int64)
        m = positions < ne
        out[m] = head[positions[m]]
        if np.any(~m):
            # the j-th column absent from the head is j + #{i : hs[i] - i <= j}
            hs = np.sort(head)
            gaps = hs - np.arange(ne)
            j = positions[~m] - ne
            out[~m] = j + np.searchsorted(gaps, j, side="right")
        return out

    def uncovered_entries(self, uncovered):
        """(block, position) of every uncovered entry, sorted by block then
        position."""
        live = uncovered[self.ids]
        return self.blk[live], self.pos[live]

    def first_chunks(self, blk, pos):
        """First uncovered 16-column chunk of every block (0 if none)."""
        first = np.zeros(self.n_blk, dtype=np.int64)
        if len(blk):
            # blk is sorted: each block's first entry starts its run
            starts = np.flatnonzero(np.concatenate([[True], blk[1:] != blk[:-1]]))
            first[blk[starts]] = pos[starts] // 16
        return first

    def block_position_counts(self, b, uncovered):
        """Uncovered entries per position of block b's order (length = the
        block's non-empty column count, at least 1)."""
        s, e = self.bptr[b], self.bptr[b + 1]
        live = uncovered[self.ids[s:e]]
        return np.bincount(self.pos[s:e][live], minlength=max(1, int(self.extent[b])))

    def tile_entries(self, b, k0, k1, uncovered=None):
        """Entries of block b in positions [k0, k1]: (local row, local col, id)."""
        s, e = self.bptr[b], self.bptr[b + 1]
        pos = self.pos[s:e]
        m = (pos >= k0) & (pos <= k1)
        ids = self.ids[s:e][m]
        if uncovered is not None:
            keep = uncovered[ids]
            ids = ids[keep]
            m2 = np.nonzero(m)[0][keep]
        else:
            m2 = np.nonzero(m)[0]
        lr = self.prow[s:e][m2] - b * self.bs
        lc = pos[m2] - k0
        return lr, lc, ids

    def space(self):
        return OpSpace(op_id=self.op_id, template=TC if self.op_type == "spmm" else TC_SDDMM,
                       i_perm=self.i_perm, k_perm=np.arange(self.pat.K, dtype=np.int64),
                       idx_reordered=(self.reordered, False, False),
                       blk_k_vals=_LazyKvals(self), TC_k_notsorted=self.k_notsorted)


class _BlockOrder:
    """Column order of one block, evaluated only at the requested positions
    (integer, integer array or slice)."""

    def __init__(self, op: TcOp, b):
        self.op, self.b = op, int(b)

    def __len__(self):
        return self.op.pat.K

    def __getitem__(self, idx):
        if isinstance(idx, slice):
            idx = np.arange(*idx.indices(len(self)))
        scalar = np.ndim(idx) == 0
        out = self.op.kvals(self.b, np.atleast_1d(idx))
        return out[0] if scalar else out

    def __array__(self, dtype=None, copy=None):
        return self.op.kvals(self.b, np.arange(len(self)))


class _LazyKvals(dict):
    """``blk_k_vals[b]``: the column order of block b (non-empty columns,
    then the empty ones ascending), evaluated lazily."""

    def __init__(self, op: TcOp):
        super().__init__()
        self.op = op

    def __missing__(self, b):
        v = _BlockOrder(self.op, b)
        self[b] = v
        return v


# ---------------------------------------------------------------------------
# 1D SDDMM operator
# ---------------------------------------------------------------------------
class OneDOp:
    """Nonzeros of the covered-entry subset in CSR order, cut into chunks of
    ``mbs`` (get_1D_position_space :1128-1160)."""

    def __init__(self, pat: Pattern, ids, mbs, op_id):
        self.pat = pat
        self.op_id = op_id
        self.mbs = mbs
        self.ids = np.sort(np.asarray(ids, dtype=np.int64))
        self.n = len(self.ids)
        self.n_chunks = math.ceil(self.n / mbs) if self.n else 0
        self._rc = None

    def chunk_uncovered(self, uncovered):
        live = uncovered[self.ids].astype(np.int64)
        if self.n == 0:
            return np.zeros(0, np.int64)
        return np.add.reduceat(live, np.arange(0, self.n, self.mbs))

    def row_col_nums(self):
        if self._rc is None:
            pad = self.n_chunks * self.mbs - self.n
            rows = self.pat.row_of[self.ids]
            cols = self.pat.indices[self.ids]
            rows = np.concatenate([rows, np.full(pad, rows[-1])]).reshape(-1, self.mbs)
            cols = np.concatenate([cols, np.full(pad, cols[-1])]).reshape(-1, self.mbs)
            rs = np.sort(rows, axis=1)
            cs = np.sort(cols, axis=1)
            rn = 1 + np.count_nonzero(np.diff(rs, axis=1), axis=1)
            cn = 1 + np.count_nonzero(np.diff(cs, axis=1), axis=1)
            self._rc = (rn, cn)
        return self._rc

    def space(self):
        rows = self.pat.row_of[self.ids]
        return OpSpace(op_id=self.op_id, template=ONE_D, i_perm=np.arange(self.pat.M, dtype=np.int64),
                       k_perm=np.arange(self.pat.K, dtype=np.int64), idx_reordered=(False, False, False),
                       ori_row_ids_1d=rows, ori_col_ids_1d=self.pat.indices[self.ids], nnz_id_1d=self.ids)


# ---------------------------------------------------------------------------
# search state
# ---------------------------------------------------------------------------
class _Sel:
    """A selected (or candidate) tile during the search."""
    __slots__ = ("op", "kind", "ts", "pos", "atomic", "pred_cost", "nnz_unc", "j_num", "cov_ids",
                 "cov_rows", "cov_cols", "cov_shape", "i_rng", "k_rng", "best_ts", "params",
                 "pred_avg", "nnz0")

    def __init__(self, **kw):
        for k in self.__slots__:
            setattr(self, k, kw.get(k))


def _sum_pred(tiles):
    s = 0
    for t in tiles:
        s = s + t.pred_cost
    return s


class SpmmPlanner:
    def __init__(self, A, N, cost: CostModel = A100_FP16, max_bucket_size=None, only_TC=False,
                 only_ELL=False, max_avg_cost_diff=0.2, penalty=1, max_level_num=float("inf"),
                 single_level=False, no_withdraw=False, tc_k_notsorted=False, reorder_k_by_nnz=True):
        self.pat = Pattern(A)
        self.N = int(N)
        self.tc_k_notsorted = bool(tc_k_notsorted)
        self.k_by_count = bool(reorder_k_by_nnz)
        self.tc_sizes = tc_tile_sizes("spmm", self.tc_k_notsorted)
        self.cost = cost
        self.mbs = max_bucket_size or estimate_max_bucket_size(self.pat.nnz, cost.sm_num)
        self.only_TC, self.only_ELL = only_TC, only_ELL
        self.max_avg_cost_diff = float("inf") if only_ELL else max_avg_cost_diff
        self.penalty = penalty
        self.max_level_num = max_level_num
        self.single_level = single_level
        self.no_withdraw = no_withdraw
        self.dsize = cost.dsize
        self.j_num = min(32, self.N)
        self.uncovered = np.ones(self.pat.nnz, dtype=bool)
        self._upd_cache = {}
        self._tc_unc = None

    # ---------------- candidate operators ----------------
    def _level1(self):
        pat = self.pat
        self.ell_ops = [EllOp(pat, np.arange(pat.nnz), self.mbs, 0)] if not self.only_TC else []
        nid = 2
        self.tc = None
        if not self.only_ELL:
            ident = np.arange(pat.M, dtype=np.int64)
            by_len = np.argsort(-pat.row_nnz, kind="stable")
            kw = dict(k_notsorted=self.tc_k_notsorted, k_by_count=self.k_by_count)
            cands = [TcOp(pat, ident, nid, **kw)]
            if not np.array_equal(by_len, ident):
                cands.append(TcOp(pat, by_len, nid, **kw))
            best, bd = None, 0
            for c in cands:
                d = c.density()
                if d > bd:
                    best, bd = c, d
            self.tc = best if best is not None else cands[0]
            nid += 1
        self.next_id = nid
        if self.only_TC:
            # the reference still builds the level-1 ELL operator (ids 0, 1)
            # but does not search it
            self.level1_ell = EllOp(pat, np.arange(pat.nnz), self.mbs, 0)
        else:
            self.level1_ell = self.ell_ops[0]

    def _next_level_ops(self, TC_is):
        """gen_full_next_level_subops (:1051-1094): the uncovered elements,
        split into rows touched by tensor-core tiles and the others, each
        becomes a new ELL operator (ids advance by two per operator: ELL and
        the unused CSR variant)."""
        unc = np.nonzero(self.uncovered)[0]
        rows = self.pat.row_of[unc]
        aff = TC_is[rows]
        ops = []
        for part in (unc[aff], unc[~aff]):
            ops.append(EllOp(self.pat, part, self.mbs, self.next_id))
            self.next_id += 2
        return ops

    # ---------------- costs ----------------
    def _ell_shapes(self, op):
        return op.tile_shapes(self.N)

    def ell_lower_bound(self):
        return self.cost.ell_lower_bound(self._ell_shapes(self.level1_ell))

    # ---------------- ELL search ----------------
    def _search_ell(self, ops, best_avg):
        """search_best_tile_given_op_BSPMM (:728-835) over all ops."""
        best = None
        self._ell_cache = {}
        ori_rn = self.pat.row_nnz
        for op in ops:
            upd = self._upd(op)
            indptr_u = np.concatenate([[0], np.cumsum(upd)])
            for (I, J, K) in self._ell_shapes(op):
                tl = op.valid_positions(I, K)
                sb = op.short_begin
                rest_orig = ori_rn[op.i_perm[op.hyb_new_rows[sb:]]]
                rest_upd = upd[sb:]
                arows = np.nonzero((rest_orig > rest_upd) & (rest_upd > 0))[0] + sb
                apos = np.concatenate([np.arange(((sb - 1) // I) + 1), arows // I])
                tile_pos_is = [p for p in tl]
                apos = np.intersect1d(tile_pos_is, apos)
                napos = np.setdiff1d(tile_pos_is, apos, assume_unique=True)
                entry = []
                for pos_is, atomic in ((apos, True), (napos, False)):
                    pos_is = np.asarray(pos_is, dtype=np.int64)
                    if len(pos_is) == 0:
                        entry.append((pos_is, atomic, None, np.array([])))
                        continue
                    s = indptr_u[I * pos_is]
                    e = indptr_u[np.minimum(I * (pos_is + 1), len(indptr_u) - 1)]
                    nn = e - s
                    keep = nn > 0
                    pos_is = pos_is[keep]
                    nn = nn[keep] * J
                    if len(pos_is) == 0:
                        entry.append((pos_is, atomic, nn, np.array([])))
                        continue
                    k_is = op.k_is(I, K, pos_is)
                    mlp = getattr(self.cost, "mlp", None)
                    if mlp is not None:
                        # learned model: every candidate of this shape in one
                        # inference launch, from the uncovered row counts
                        rows = I * pos_is[:, None] + np.arange(I)[None, :]
                        rn = np.where(rows < len(upd), upd[np.minimum(rows, len(upd) - 1)], 0)
                        costs = mlp.ell_costs(I, K, rn, k_is, self.N, atomic)
                    else:
                        costs = self.cost.ell_costs(I, J, K, k_is, atomic)
                    entry.append((pos_is, atomic, nn, costs))
                    with np.errstate(divide="ignore", invalid="ignore"):
                        avg = costs / nn
                    idx = int(np.nanargmin(avg))
                    if avg[idx] < best_avg:
                        best_avg = avg[idx]
                        best = (op, (I, J, K), int(pos_is[idx]), atomic, int(nn[idx]))
                self._ell_cache[(op.op_id, (I, J, K))] = entry
        if best is None:
            return None, best_avg
        op, shp, pos, atomic, nn = best
        t = self._ell_tile(op, shp, pos, atomic)
        t.pred_cost = nn * best_avg
        t.pred_avg = t.pred_cost / np.float32(t.nnz_unc)
        return t, best_avg

    def _upd(self, op):
        key = op.op_id
        if key not in self._upd_cache:
            self._upd_cache[key] = op.upd_rows(self.uncovered)[0]
        return self._upd_cache[key]

    def _ell_tile(self, op, shp, pos, atomic):
        I, J, K = shp
        r0 = I * pos
        r1 = min(I * (pos + 1), op.n_folded) - 1
        upd = self._upd(op)
        nnz_unc = self.j_num * int(upd[r0:r1 + 1].sum())
        ts = ((None, I), (None, J), (1, K))
        return _Sel(op=op, kind=ELL, ts=ts, pos=(int(pos), 0, 0), atomic=atomic, nnz_unc=nnz_unc,
                    j_num=self.j_num, i_rng=(r0, r1), best_ts=([None, I, 1], [None, J // 32, 32], (1, K)),
                    params={"use_implicit_unroll": True, "last_bucket": K == self.mbs})

    def _local_search_ell(self, sel, target, TC_row_tile_dict, TC_row_costs, n_before, reverse_idx):
        """local_search_ELL (:1410-1478)."""
        op = sel.op
        I, J, K = sel.ts[0][1], sel.ts[1][1], sel.ts[2][1]
        good = []
        for pos_is, atomic, nn, costs in self._ell_cache[(op.op_id, (I, J, K))]:
            if len(pos_is) == 0:
                continue
            with np.errstate(divide="ignore", invalid="ignore"):
                avg = costs / nn
            gi = avg <= target
            for cost, p in zip(costs[gi], pos_is[gi]):
                t = self._ell_tile(op, (I, J, K), int(p), atomic)
                t.pred_cost = cost
                t.pred_avg = t.pred_cost / np.float32(t.nnz_unc)
                t.best_ts = sel.best_ts
                t.params = sel.params
                good.append(t)
                rows = op.hyb_new_rows[np.arange(p * I, min((p + 1) * I, op.n_folded))]
                rows = op.i_perm[rows]
                blk_rows = reverse_idx[rows] // 16
                if len(np.unique(blk_rows)) == 1:
                    b = int(blk_rows[0])
                    TC_row_tile_dict[b] = np.concatenate([TC_row_tile_dict[b], [n_before + len(good) - 1]])
                    TC_row_costs[b] = TC_row_costs[b] + cost
        return good

    # ---------------- tensor-core search ----------------
    def _tc_tile(self, b, ts, kpos, atomic, uncovered_only):
        tc = self.tc
        Kt = ts[2][1]
        r0 = 16 * b
        r1 = min(16 * (b + 1), self.pat.M) - 1
        k0 = int(Kt * kpos)
        k1 = min(int(Kt * (kpos + 1)), self.pat.K) - 1
        return _Sel(op=tc, kind=TC, ts=ts, pos=(int(b), 0, kpos), atomic=atomic, j_num=self.j_num,
                    i_rng=(r0, r1), k_rng=(k0, k1), best_ts=ts, params=dict(TC_PARAMS))

    def _tc_nnz(self, t, uncovered):
        lr, lc, ids = self.tc.tile_entries(t.pos[0], t.k_rng[0], t.k_rng[1], uncovered)
        return len(ids)

    def _tc_uncovered(self):
        """Uncovered tensor-core entries: (block, position, each block's
        first uncovered 16-column chunk, per (block, chunk relative to it)
        the code b * span16 + chunk and its entry count, span16), kept until
        the uncovered set changes."""
        if self._tc_unc is None:
            blk, pos = self.tc.uncovered_entries(self.uncovered)
            first = self.tc.first_chunks(blk, pos)
            if self.single_level:
                first = first * 0
            rel = pos // 16 - first[blk]
            span16 = int(rel.max()) + 1 if len(rel) else 1
            # entries come sorted by (block, position), so the codes are
            # nondecreasing and their runs are np.unique's groups
            c16, n16 = _run_counts(blk * span16 + rel)
            self._tc_unc = (blk, pos, first, c16, n16, span16)
        return self._tc_unc

    def _tc_windows(self, w):
        """(codes b * span + window, entry counts, span) of the uncovered
        entries in windows of w 16-column chunks from each block's first
        uncovered chunk, summed from the per-chunk counts."""
        blk, pos, first, c16, n16, span16 = self._tc_uncovered()
        b16, r16 = c16 // span16, c16 % span16
        win = r16 // w
        span = int(win.max()) + 1
        code2 = b16 * span + win
        starts = np.flatnonzero(np.concatenate([[True], code2[1:] != code2[:-1]]))
        return code2[starts], np.add.reduceat(n16, starts), span

    def _search_tc_op(self, TC_row_costs):
        """search_best_TC_tile_given_op (:558-696): best atomic tile over
        windows aligned to every block's first uncovered chunk, and the best
        whole-row (owned, withdraw) alternative."""
        tc = self.tc
        blk, pos, first = self._tc_uncovered()[:3]
        tot = np.bincount(blk, minlength=tc.n_blk)
        best_key, best_cost = None, float("inf")
        for ts in self.tc_sizes:
            Kt = ts[2][1]
            w = Kt // 16
            if len(blk):
                code, cnt, span = self._tc_windows(w)
                mp = int(np.argmax(cnt))
                r, c = int(code[mp] // span), int(code[mp] % span)
                cost = self.cost.tc_cost(Kt, True, self.penalty)
                pavg = cost / cnt[mp] / ts[1][1]
                kpos = c + first[r] * Fraction(16, Kt)
                if pavg < best_cost:
                    best_cost = pavg
                    best_key = (ts, [(r, kpos)], True)
            nonempty = tc.blk_nums[ts]
            no_atomic = self.cost.tc_cost(Kt, False, self.penalty)
            extra = no_atomic * nonempty - TC_row_costs
            if self.no_withdraw:
                extra = no_atomic * nonempty
            with np.errstate(divide="ignore", invalid="ignore"):
                pavgs = extra / tot / ts[1][1]
            if np.all(np.isnan(pavgs)):
                continue
            mr = int(np.nanargmin(pavgs))
            mc = np.nanmin(pavgs)
            if mc < best_cost:
                best_cost = mc
                best_key = (ts, [(mr, i) for i in tc.row_positions(ts, mr)], False)
        return best_key, best_cost

    def _search_tc_block(self, b, counts, selected_row, best_possible_ell):
        """search_best_TC_tile_given_csr (:403-542) for one block."""
        tc = self.tc
        # chunk sums over the block's non-empty prefix (all later chunks of
        # the reference's full-length order are empty and never win)
        L = math.ceil(len(counts) / 16)
        padc = np.zeros(L * 16, dtype=np.int64)
        padc[:len(counts)] = counts
        base = padc.reshape(L, 16).sum(axis=1)
        nchunk = L
        tot = int(base.sum())
        cs = np.concatenate([[0], np.cumsum(base)])
        best_key, best_cost = None, float("inf")
        unit = {}
        sel_pred = _sum_pred(selected_row)
        if not self.single_level:
            # entries in the window of w chunks from every chunk, for all
            # tile widths at once (windows end at the block's last chunk)
            ws = np.asarray([ts[2][1] // 16 for ts in self.tc_sizes])
            per_all = cs[np.minimum(np.arange(L)[None, :] + ws[:, None], L)] - cs[None, :L]
            mps = np.argmax(per_all, axis=1)
        for n, ts in enumerate(self.tc_sizes):
            Kt = ts[2][1]
            w = Kt // 16
            if self.single_level:
                per = np.add.reduceat(base, np.arange(0, nchunk, w))
                mp = int(np.argmax(per))
            else:
                per = per_all[n]
                mp = int(mps[n])
            cost = self.cost.tc_cost(Kt, True, self.penalty)
            unit[ts] = [None, cost]
            with np.errstate(divide="ignore", invalid="ignore"):
                pavg = cost / per[mp] / ts[1][1]
            if pavg < best_cost and pavg < best_possible_ell:
                best_cost = pavg
                best_key = (ts, [mp if self.single_level else mp * Fraction(16, Kt)], True)
            nonempty = int(tc.blk_nums[ts][b])
            no_atomic = self.cost.tc_cost(Kt, False, self.penalty)
            unit[ts][0] = no_atomic
            extra = no_atomic * nonempty - sel_pred
            if self.no_withdraw:
                extra = no_atomic * nonempty
            pavgs = extra / tot / ts[1][1]
            if pavgs < best_cost and pavgs < best_possible_ell:
                best_cost = pavgs
                best_key = (ts, tc.row_positions(ts, b), False)
        return best_key, best_cost, unit

    def _local_tc_block(self, b, counts, ts, target, no_atomic, atomic_cost, selected_row):
        """local_search_TC_tiles_given_csr (:1117-1210)."""
        Kt = ts[2][1]
        nz = np.nonzero(counts)[0]
        neb = int(nz[0]) // 16
        if self.single_level:
            neb = 0
        # windows of Kt from the first uncovered chunk; windows past the
        # block's non-empty prefix are empty and never selected
        nwin = max(1, math.ceil((len(counts) - neb * 16) / Kt))
        full = np.zeros(neb * 16 + nwin * Kt, dtype=np.int64)
        full[:len(counts)] = counts
        nnz_upd = full[neb * 16:].reshape(nwin, Kt).sum(axis=1)
        nonempty = int(self.tc.blk_nums[ts][b])
        extra = no_atomic * nonempty - _sum_pred(selected_row)
        if self.no_withdraw:
            extra = no_atomic * nonempty
        pavg = extra / np.sum(nnz_upd) / ts[1][1]
        if pavg <= target:
            out = []
            for i in self.tc.row_positions(ts, b):
                t = self._tc_tile(b, ts, i, False, False)
                t.pred_cost = no_atomic
                out.append(t)
            return out
        kbeg = neb * Fraction(16, Kt)
        out = []
        for i in np.nonzero(atomic_cost <= nnz_upd * ts[1][1] * target)[0]:
            t = self._tc_tile(b, ts, int(i) + kbeg, True, True)
            t.pred_cost = atomic_cost
            out.append(t)
        return out

    def _local_tc_op(self, sel, target, TC_row_tile_dict, TC_row_costs, n_before, TC_is):
        """local_search_TC_tiles (:1213-1405): whole rows (owned tiles of
        the best width per row) whose withdraw cost is within target, then
        every atomic tile of the selected width within target."""
        tc = self.tc
        ts = sel.ts
        Kt = ts[2][1]
        blk, pos, first = self._tc_uncovered()[:3]
        tot = np.bincount(blk, minlength=tc.n_blk)
        tsl = self.tc_sizes
        nonempty = np.asarray([tc.blk_nums[t] for t in tsl])
        no_atomic = np.asarray([self.cost.tc_cost(t[2][1], False, self.penalty) for t in tsl])
        extra = no_atomic.reshape(-1, 1) * nonempty - TC_row_costs
        if self.no_withdraw:
            extra = no_atomic.reshape(-1, 1) * nonempty
        cand = np.nanargmin(extra, axis=0)
        with np.errstate(divide="ignore", invalid="ignore"):
            rowavg = np.nanmin(extra, axis=0) / tot / sel.j_num
        sel_rows = np.nonzero(rowavg <= target)[0]
        TC_row_costs[sel_rows] = -1
        good = []
        for r in sel_rows:
            t_ts = tsl[cand[r]]
            for i in tc.row_positions(t_ts, int(r)):
                t = self._tc_tile(int(r), t_ts, i, False, False)
                t.pred_cost = no_atomic[cand[r]]
                t.best_ts = t_ts
                good.append(t)
        for r in sel_rows:
            TC_is[r * 16:min((r + 1) * 16, self.pat.M)] = True
        atomic_cost = self.cost.tc_cost(Kt, True, self.penalty)
        poses = []
        if len(blk):
            code, cnt, span = self._tc_windows(Kt // 16)
            ok = atomic_cost / cnt / sel.j_num <= target
            sel_set = set(int(x) for x in sel_rows)
            for cd in code[ok]:
                r, i = int(cd // span), int(cd % span)
                if r not in sel_set:
                    poses.append((r, i + first[r] * Fraction(16, Kt)))
        rows, counts = np.unique([p[0] for p in poses], return_counts=True)
        start = n_before + len(good)
        for r, num in zip(rows, counts):
            TC_row_tile_dict[r] = np.concatenate([TC_row_tile_dict[r], np.arange(start, start + num)])
            TC_row_costs[r] = TC_row_costs[r] + atomic_cost * num
            start += num
            TC_is[r * 16:(r + 1) * 16] = True
        good2 = []
        for r, kp in poses:
            t = self._tc_tile(r, ts, kp, True, True)
            t.pred_cost = atomic_cost
            good2.append(t)
        return good + good2

    # ---------------- selection bookkeeping ----------------
    def _finalise(self, t, ref_uncovered=None):
        """update_tile_after_selection: record the entries the tile covers
        (those still uncovered, or all of ``ref_uncovered``'s)."""
        unc = self.uncovered if ref_uncovered is None else ref_uncovered
        if t.kind == TC:
            lr, lc, ids = self.tc.tile_entries(t.pos[0], t.k_rng[0], t.k_rng[1], unc)
            t.cov_rows, t.cov_cols, t.cov_ids = lr, lc, ids
            t.cov_shape = (t.i_rng[1] - t.i_rng[0] + 1, t.k_rng[1] - t.k_rng[0] + 1)
        else:
            op = t.op
            r0, r1 = t.i_rng
            s, e = op.indptr[r0], op.indptr[r1 + 1]
            ids = op.ids[s:e]
            keep = unc[ids]
            rows = (op.frow[s:e] - r0)[keep]
            t.cov_rows, t.cov_cols, t.cov_ids = rows, op.cols[s:e][keep], ids[keep]
            t.cov_shape = (r1 - r0 + 1, self.pat.K)
        t.nnz0 = len(t.cov_ids)

    def _cover(self, tiles):
        for t in tiles:
            self.uncovered[t.cov_ids] = False
        self._upd_cache = {}
        self._tc_unc = None

    # ---------------- main ----------------
    def search(self):
        self._level1()
        pat = self.pat
        M = pat.M
        selected = []
        TC_row_num = math.ceil(M / 16)
        TC_row_tile_dict = {i: np.zeros(0, dtype=np.int64) for i in range(TC_row_num)}
        TC_row_costs = np.full(TC_row_num, 0.0)
        TC_is = np.full(M, False)
        reverse_idx = np.argsort(self.tc.i_perm) if self.tc is not None else np.arange(M)
        best_possible_ell = self.ell_lower_bound() if self.ell_ops else float("inf")
        all_subops = list(self.ell_ops) if not self.only_TC else []
        level_num = 1

        if self.tc is not None and all_subops and not self.only_TC and not self.only_ELL:
            selected = self._tc_rows_pass(best_possible_ell, TC_row_tile_dict, TC_row_costs, TC_is)
            if not self.single_level:
                all_subops = self._next_level_ops(TC_is)

        stall = 0
        guard = 0
        while self.uncovered.any():
            guard += 1
            if guard > 100000:
                raise RuntimeError("format search did not converge")
            good_tc = []
            if self.tc is not None:
                key, best_tc = self._search_tc_op(TC_row_costs)
                if key is not None:
                    ts, poses, atomic = key
                    for (b, kp) in poses:
                        t = self._tc_tile(int(b), ts, kp, atomic, atomic)
                        if atomic:
                            t.nnz_unc = self.j_num * self._tc_nnz(t, self.uncovered)
                        else:
                            t.nnz_unc = self.j_num * self._tc_nnz(t, None)
                        t.pred_cost = best_tc * t.nnz_unc
                        with np.errstate(divide="ignore", invalid="ignore"):
                            t.pred_avg = t.pred_cost / np.float32(t.nnz_unc)
                        good_tc.append(t)
            init_avg = good_tc[0].pred_avg if good_tc else float("inf")
            chosen = good_tc
            if not (init_avg < best_possible_ell) and all_subops:
                t, _ = self._search_ell(all_subops, init_avg)
                if t is not None:
                    chosen = [t]
            if len(chosen) == 0:
                stall += 1
                if stall == 2:
                    raise RuntimeError("no tile can cover the remaining elements")
                all_subops = self._next_level_ops(TC_is)
                continue
            stall = 0
            best_avg = chosen[0].pred_avg
            target = best_avg * (1 + self.max_avg_cost_diff) if best_avg >= 0 else \
                best_avg * (1 - self.max_avg_cost_diff)
            if chosen[0].kind == TC:
                good = self._local_tc_op(chosen[0], target, TC_row_tile_dict, TC_row_costs, len(selected), TC_is)
                J = chosen[0].ts[1][1]
                if not good and self.j_num < J:
                    # the search ranks tensor-core tiles per J = 32 columns
                    # of B (tile_sizes[1][1], my_branch_and_bound.py:531,
                    # :683) and the local search per min(N, 32) columns
                    # (selected_tile.j_num, :1322, :1374); for N < 32 the
                    # chosen tile fails its own window and the reference's
                    # loop never ends.  Widen the window by J / j_num, which
                    # puts both on one scale (an empty result changed
                    # nothing, so the retry starts from the same state).
                    good = self._local_tc_op(chosen[0], target * J / self.j_num, TC_row_tile_dict,
                                             TC_row_costs, len(selected), TC_is)
            else:
                good = self._local_search_ell(chosen[0], target, TC_row_tile_dict, TC_row_costs,
                                              len(selected), reverse_idx)
            for t in good:
                self._finalise(t)
            selected.extend(good)
            self._cover(good)
            if not self.uncovered.any():
                break
            nxt = level_num < self.max_level_num and chosen[0].kind == TC
            if self.single_level:
                nxt = level_num < 1
            if nxt:
                level_num += 1
                all_subops = self._next_level_ops(TC_is)
        self.level_num = level_num
        return self._post_process(selected, TC_row_tile_dict, TC_row_costs, reverse_idx)

    def _tc_rows_pass(self, best_possible_ell, TC_row_tile_dict, TC_row_costs, TC_is):
        """search_TC_tiles_only_by_rows (:238-389): blocks are independent;
        in each, repeatedly take the best tile (or the whole row of owned
        tiles), widened by the block-local search, until the block is covered
        or no tile beats the best possible ELL cost."""
        tc = self.tc
        selected = []
        start_uncovered = self.uncovered.copy()
        for b in range(tc.n_blk):
            counts = tc.block_position_counts(b, self.uncovered)
            row_sel = []
            while counts.sum() > 0:
                key, best_cost, unit = self._search_tc_block(b, counts, row_sel, best_possible_ell)
                if best_cost == float("inf"):
                    break
                ts, poses, atomic = key
                # The reference widens by best * (1 + diff) here
                # (my_branch_and_bound.py:300).  A whole-row option whose
                # withdraw cost is negative (the row's earlier atomic tiles
                # cost more than owning the row) then gets a window below
                # the best itself, the local search returns nothing and the
                # block never changes: the reference's loop does not end.
                # The sign-aware window of its main loop (:1563-1568) keeps
                # the best inside and changes no plan that terminates.
                target = best_cost * (1 + self.max_avg_cost_diff) if best_cost >= 0 else \
                    best_cost * (1 - self.max_avg_cost_diff)
                good = self._local_tc_block(b, counts, ts, target, unit[ts][0], unit[ts][1], row_sel)
                if not good:
                    break  # nothing selected: the later passes cover the rest
                if good and not good[0].atomic:
                    row_sel = good
                    ref = start_uncovered
                else:
                    row_sel = row_sel + good
                    ref = self.uncovered
                for t in good:
                    self._finalise(t, ref)
                for t in good:
                    lr, lc, ids = tc.tile_entries(b, t.k_rng[0], t.k_rng[1], self.uncovered)
                    self.uncovered[ids] = False
                counts = tc.block_position_counts(b, self.uncovered)
            selected.extend(row_sel)
            if row_sel and not row_sel[0].atomic:
                TC_row_costs[b] = -1
            else:
                TC_row_tile_dict[b] = np.arange(len(selected) - len(row_sel), len(selected))
                TC_row_costs[b] = _sum_pred(row_sel)
            if row_sel:
                TC_is[b * 16:(b + 1) * 16] = True
        self._upd_cache = {}
        self._tc_unc = None
        return selected

    # ---------------- withdraw post-processing ----------------
    def _post_process(self, selected, TC_row_tile_dict, TC_row_costs, reverse_idx):
        """post_process_for_withdraw_BSPMM (:1652-1702)."""
        M = self.pat.M
        whole = np.nonzero(TC_row_costs == -1)[0]
        to_del = np.concatenate([TC_row_tile_dict[b] for b in whole] + [np.zeros(0)]).astype(np.int64)
        remain_idx = np.setdiff1d(np.arange(len(selected)), to_del, assume_unique=True)
        remains = [selected[i] for i in remain_idx]
        tiles = []
        spaces = {}
        ori_rn = self.pat.row_nnz

        def space_of(op):
            if op.op_id not in spaces:
                spaces[op.op_id] = op.space()
            return spaces[op.op_id]

        everything = np.ones(self.pat.nnz, dtype=bool)
        for t in remains:
            if t.kind == TC:
                if not t.atomic:
                    self._finalise(t, everything)
                cov = _tile_csr(t.cov_rows, t.cov_cols, t.cov_shape)
                nt = Tile(op=space_of(t.op), tile_sizes=t.ts, tile_pos=t.pos, params=dict(TC_PARAMS),
                          best_tile_sizes=t.best_ts, best_params=dict(TC_PARAMS), is_atomic=bool(t.atomic),
                          tile_i_rng=t.i_rng, tile_k_rng=None,
                          k_vals=np.arange(t.k_rng[0], t.k_rng[1] + 1, dtype=np.int64), covered=cov,
                          pred_cost=float(t.pred_cost), nnz_when_selected=int(self.j_num * len(t.cov_ids)),
                          j_num=self.j_num)
                nt.cov_ids = t.cov_ids
                tiles.append(nt)
            else:
                op = t.op
                r0, r1 = t.i_rng
                out_rows = op.i_perm[op.hyb_new_rows[r0:r1 + 1]]
                rows = reverse_idx[out_rows] // 16
                ur, idx = np.unique(rows, return_inverse=True)
                inter, _, y_ind = np.intersect1d(whole, ur, assume_unique=True, return_indices=True)
                i_vals = out_rows.copy()
                atomic = bool(t.atomic)
                cov_nnz_rows = np.bincount(t.cov_rows, minlength=r1 - r0 + 1)
                if len(inter) > 0:
                    hit = np.zeros(len(out_rows), dtype=bool)
                    for i in y_ind:
                        hit |= idx == i
                    rr = np.nonzero(hit)[0]
                    i_vals[rr] = M
                    if atomic:
                        rest = np.setdiff1d(np.arange(len(out_rows)), rr, assume_unique=True)
                        if ori_rn[out_rows[rest]].sum() == cov_nnz_rows[rest].sum():
                            atomic = False
                if not atomic:
                    i_vals[cov_nnz_rows == 0] = M
                cov = _tile_csr(t.cov_rows, t.cov_cols, (r1 - r0 + 1, self.pat.K))
                nt = Tile(op=space_of(op), tile_sizes=t.ts, tile_pos=t.pos, params=t.params,
                          best_tile_sizes=t.best_ts, best_params=t.params, is_atomic=atomic,
                          tile_i_rng=None, tile_k_rng=None, i_vals=i_vals, covered=cov,
                          pred_cost=float(t.pred_cost), nnz_when_selected=int(self.j_num * len(t.cov_ids)),
                          j_num=self.j_num)
                nt.cov_ids = t.cov_ids
                tiles.append(nt)
        return Plan(op_type="spmm", shape=(self.pat.M, self.pat.K), tiles=tiles, max_bucket_size=self.mbs,
                    level_num=self.level_num, meta={"cost_model": self.cost.name})


def search_spmm(A, N, cost: CostModel = A100_FP16, **kw) -> Plan:
    """Select a hybrid tile plan for C = A @ B with B of N columns."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        return SpmmPlanner(A, N, cost=cost, **kw).search()


# ---------------------------------------------------------------------------
# SDDMM
# ---------------------------------------------------------------------------
class SddmmPlanner:
    """SDDMM branch of the same search: 1D nonzero-chunk tiles against
    16x16 tensor-core blocks (gen_candidate_formats_BSDDMM :1837-1900; the
    SDDMM paths of search_best_TC_tile_given_csr / _given_op,
    local_search_TC_tiles*, search_best_tile_given_op_BSDDMM,
    local_search_1D_BSDDMM; post_process_for_withdraw_BSDDMM :1709-1751)."""

    def __init__(self, A, F, cost: CostModel = A100_FP16, max_bucket_size=32, only_TC=False, only_ELL=False,
                 max_avg_cost_diff=0.2, max_level_num=float("inf"), single_level=False, tc_k_notsorted=False,
                 reorder_k_by_nnz=True):
        self.pat = Pattern(A)
        self.F = int(F)
        self.tc_k_notsorted = bool(tc_k_notsorted)
        self.k_by_count = bool(reorder_k_by_nnz)
        self.cost = cost
        self.mbs = max_bucket_size
        self.only_TC, self.only_ELL = only_TC, only_ELL
        self.max_avg_cost_diff = float("inf") if (only_TC or only_ELL) else max_avg_cost_diff
        self.max_level_num = max_level_num
        self.single_level = single_level
        self.uncovered = np.ones(self.pat.nnz, dtype=bool)
        js = [j for j in (16, 32, 64) if j <= self.F]
        self.tile_j = max(js) if js else None
        if self.tc_k_notsorted:
            self.tile_j = tc_tile_sizes("sddmm", True)[0][1][1]

    def _ts(self):
        return ((None, 16), (None, self.tile_j), (None, 16))

    def _tc_cost(self):
        return self.cost.tc_sddmm_cost(self.tile_j, 16)

    def _scale(self):
        return math.ceil(self.F / self.tile_j)

    def search(self):
        pat = self.pat
        F = self.F
        oned = OneDOp(pat, np.arange(pat.nnz), self.mbs, 0)
        tc = None
        nid = 1
        if not self.only_ELL and self.tile_j is not None:
            ident = np.arange(pat.M, dtype=np.int64)
            by_len = np.argsort(-pat.row_nnz, kind="stable")
            kw = dict(op_type="sddmm", k_notsorted=self.tc_k_notsorted, k_by_count=self.k_by_count)
            cands = [TcOp(pat, ident, nid, **kw)]
            if not np.array_equal(by_len, ident):
                cands.append(TcOp(pat, by_len, nid, **kw))
            best, bd = None, 0
            for c in cands:
                d = c.density()
                if d > bd:
                    best, bd = c, d
            tc = best if best is not None else cands[0]
            nid += 1
        self.tc = tc
        self.next_id = nid
        all_subops = [] if self.only_TC else [oned]
        best_possible = self.cost.one_d_lower_bound(F, self.mbs) if all_subops else float("inf")
        selected = []
        level_num = 1
        if tc is not None and all_subops and not self.only_TC:
            selected = self._rows_pass(best_possible)
            if not self.single_level:
                all_subops = [self._next_1d()]
        guard = 0
        while self.uncovered.any():
            guard += 1
            if guard > 100000:
                raise RuntimeError("SDDMM format search did not converge")
            good_tc = []
            if tc is not None:
                key, best_tc = self._search_tc_op()
                if key is not None:
                    b, kp = key
                    t = self._tc_tile(b, kp)
                    t.nnz_unc = F * len(tc.tile_entries(b, t.k_rng[0], t.k_rng[1], self.uncovered)[2])
                    t.pred_cost = best_tc * t.nnz_unc
                    with np.errstate(divide="ignore", invalid="ignore"):
                        t.pred_avg = t.pred_cost / np.float32(t.nnz_unc)
                    good_tc = [t]
            init_avg = good_tc[0].pred_avg if good_tc else float("inf")
            chosen = good_tc
            if not (init_avg < best_possible) and all_subops:
                t = self._search_1d(all_subops, init_avg)
                if t is not None:
                    chosen = [t]
            if not chosen:
                raise RuntimeError("no tile can cover the remaining SDDMM elements")
            best_avg = chosen[0].pred_avg
            target = best_avg * (1 + self.max_avg_cost_diff) if best_avg >= 0 else \
                best_avg * (1 - self.max_avg_cost_diff)
            if chosen[0].kind == TC_SDDMM:
                good = self._local_tc(chosen[0], target)
            else:
                good = self._local_1d(chosen[0], target)
            for t in good:
                self._finalise(t)
            selected.extend(good)
            for t in good:
                self.uncovered[t.cov_ids] = False
            if not self.uncovered.any():
                break
            nxt = level_num < self.max_level_num and chosen[0].kind == TC_SDDMM
            if self.single_level:
                nxt = level_num < 1
            if nxt:
                level_num += 1
                all_subops = [self._next_1d()]
        return self._post_process(selected, level_num)

    # ---------------- operators / tiles ----------------
    def _next_1d(self):
        op = OneDOp(self.pat, np.nonzero(self.uncovered)[0], self.mbs, self.next_id)
        self.next_id += 1
        return op

    def _tc_tile(self, b, kpos):
        Kt = 16
        r0 = 16 * b
        r1 = min(16 * (b + 1), self.pat.M) - 1
        k0 = int(Kt * kpos)
        k1 = min(int(Kt * (kpos + 1)), self.pat.K) - 1
        return _Sel(op=self.tc, kind=TC_SDDMM, ts=self._ts(), pos=(int(b), 0, kpos), atomic=False,
                    j_num=self.F, i_rng=(r0, r1), k_rng=(k0, k1), best_ts=self._ts(), params=dict(TC_PARAMS))

    def _finalise(self, t):
        if t.kind == TC_SDDMM:
            lr, lc, ids = self.tc.tile_entries(t.pos[0], t.k_rng[0], t.k_rng[1], self.uncovered)
            t.cov_rows, t.cov_cols, t.cov_ids = lr, lc, ids
            t.cov_shape = (t.i_rng[1] - t.i_rng[0] + 1, t.k_rng[1] - t.k_rng[0] + 1)
        else:
            op = t.op
            s = t.pos[0] * self.mbs
            e = min(s + self.mbs, op.n)
            ids = op.ids[s:e]
            flags = self.uncovered[ids]
            t.cov_ids = ids[flags]
            t.cov_rows = flags.astype(np.float64)

    # ---------------- tensor-core blocks ----------------
    def _rows_pass(self, best_possible):
        tc = self.tc
        F = self.F
        cost = self._tc_cost()
        scale = self._scale()
        selected = []
        for b in range(tc.n_blk):
            counts = tc.block_position_counts(b, self.uncovered)
            while counts.sum() > 0:
                L = math.ceil(len(counts) / 16)
                padc = np.zeros(L * 16, dtype=np.int64)
                padc[:len(counts)] = counts
                base = padc.reshape(L, 16).sum(axis=1)
                mp = int(np.argmax(base))
                with np.errstate(divide="ignore", invalid="ignore"):
                    pavg = cost * scale / base[mp] / F
                if not (pavg < float("inf") and pavg < best_possible):
                    break
                target = pavg * (1 + self.max_avg_cost_diff)
                nz = np.nonzero(counts)[0]
                neb = int(nz[0]) // 16
                nwin = max(1, math.ceil((len(counts) - neb * 16) / 16))
                full = np.zeros(neb * 16 + nwin * 16, dtype=np.int64)
                full[:len(counts)] = counts
                nnz_upd = full[neb * 16:].reshape(nwin, 16).sum(axis=1)
                good = []
                for i in np.nonzero(cost * scale <= nnz_upd * F * target)[0]:
                    t = self._tc_tile(b, int(i) + neb)
                    t.pred_cost = cost * scale
                    good.append(t)
                for t in good:
                    self._finalise(t)
                for t in good:
                    self.uncovered[t.cov_ids] = False
                selected.extend(good)
                counts = tc.block_position_counts(b, self.uncovered)
        return selected

    def _search_tc_op(self):
        tc = self.tc
        blk, pos = tc.uncovered_entries(self.uncovered)
        if len(blk) == 0:
            return None, float("inf")
        first = tc.first_chunks(blk, pos)
        if self.single_level:
            first = first * 0
        win = pos // 16 - first[blk]
        span = int(win.max()) + 1
        # entries come sorted by (block, position): the codes are nondecreasing
        code, cnt = _run_counts(blk * span + win)
        mp = int(np.argmax(cnt))
        r, c = int(code[mp] // span), int(code[mp] % span)
        pavg = self._tc_cost() * self._scale() / cnt[mp] / self.F
        return (r, c + int(first[r])), pavg

    def _local_tc(self, sel, target):
        tc = self.tc
        cost = self._tc_cost()
        scale = self._scale()
        blk, pos = tc.uncovered_entries(self.uncovered)
        first = tc.first_chunks(blk, pos)
        if self.single_level:
            first = first * 0
        win = (pos - first[blk] * 16) // 16
        span = int(win.max()) + 1
        # entries come sorted by (block, position): the codes are nondecreasing
        code, cnt = _run_counts(blk * span + win)
        ok = cost * scale / cnt / self.F <= target
        good = []
        for cd in code[ok]:
            r, i = int(cd // span), int(cd % span)
            t = self._tc_tile(r, i + int(first[r]))
            t.pred_cost = cost * scale
            good.append(t)
        return good

    # ---------------- 1D chunks ----------------
    def _search_1d(self, ops, best_avg):
        best = None
        self._avg_cache = {}
        for op in ops:
            if op.n == 0:
                continue
            rn, cn = op.row_col_nums()
            costs = self.cost.one_d_costs(rn, cn, self.F, self.mbs)
            nn = op.chunk_uncovered(self.uncovered)
            with np.errstate(divide="ignore", invalid="ignore"):
                avg = costs / nn / self.F
            self._avg_cache[op.op_id] = (op, avg)
            mp = int(np.argmin(avg))
            if avg[mp] < best_avg:
                best_avg = avg[mp]
                best = (op, mp, int(nn[mp]) * self.F)
        if best is None:
            return None
        op, mp, nnz_key = best
        t = self._one_d_tile(op, mp)
        t.pred_cost = nnz_key * best_avg
        with np.errstate(divide="ignore", invalid="ignore"):
            t.pred_avg = t.pred_cost / np.float32(t.nnz_unc)
        return t

    def _one_d_tile(self, op, p, nn=None):
        """Selection record of chunk p of ``op``; ``nn`` is the operator's
        per-chunk uncovered counts when the caller already has them (they do
        not change until the selected tiles are finalised)."""
        if nn is None:
            nn = op.chunk_uncovered(self.uncovered)
        return _Sel(op=op, kind=ONE_D, ts=(self.mbs,), pos=(int(p),), atomic=False, j_num=self.F,
                    nnz_unc=self.F * int(nn[p]), best_ts=(self.mbs,), params=dict(ONE_D_PARAMS))

    def _local_1d(self, sel, target):
        op, avg = self._avg_cache[sel.op.op_id]
        good = []
        nn = op.chunk_uncovered(self.uncovered)
        for p in np.nonzero(avg <= target)[0]:
            t = self._one_d_tile(op, int(p), nn)
            t.pred_cost = avg[p] * t.nnz_unc
            good.append(t)
        return good

    # ---------------- post-processing ----------------
    def _post_process(self, selected, level_num):
        spaces = {}
        pat = self.pat
        tiles_1d, tiles_tc = [], []
        for t in selected:
            if t.op.op_id not in spaces:
                sp_ = t.op.space()
                if t.kind == TC_SDDMM:
                    inv = t.op.inv
                    sp_.nnz_id_matrix = sp.csr_matrix(
                        (np.arange(1, pat.nnz + 1), (inv[pat.row_of], pat.indices)), shape=(pat.M, pat.K))
                spaces[t.op.op_id] = sp_
            if t.kind == TC_SDDMM:
                cov = _tile_csr(t.cov_rows, t.cov_cols, t.cov_shape)
                tiles_tc.append(Tile(op=spaces[t.op.op_id], tile_sizes=t.ts, tile_pos=t.pos, params=dict(TC_PARAMS),
                                     best_tile_sizes=t.best_ts, best_params=dict(TC_PARAMS), is_atomic=False,
                                     tile_i_rng=t.i_rng, tile_k_rng=t.k_rng, covered=cov,
                                     pred_cost=float(t.pred_cost), nnz_when_selected=int(self.F * len(t.cov_ids)),
                                     j_num=self.F))
            else:
                tiles_1d.append(Tile(op=spaces[t.op.op_id], tile_sizes=t.ts, tile_pos=t.pos,
                                     params=dict(ONE_D_PARAMS), best_tile_sizes=t.best_ts,
                                     best_params=dict(ONE_D_PARAMS), is_atomic=False, covered=t.cov_rows,
                                     pred_cost=float(t.pred_cost), nnz_when_selected=int(self.F * len(t.cov_ids)),
                                     j_num=self.F))
        return Plan(op_type="sddmm", shape=(pat.M, pat.K), tiles=tiles_1d + tiles_tc, max_bucket_size=self.mbs,
                    level_num=level_num, meta={"cost_model": self.cost.name})


def search_sddmm(A, F, cost: CostModel = A100_FP16, **kw) -> Plan:
    """Select a hybrid tile plan for out = (X @ Y^T) sampled on A's pattern."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        return SddmmPlanner(A, F, cost=cost, **kw).search()


plan_spmm = search_spmm
plan_sddmm = search_sddmm
