"""Plan data model: candidate operators ("op spaces") and selected tiles.

A *plan* is the output of the format search: an ordered list of selected
tiles, each referring to the candidate operator it was cut from.  The fields
mirror what the reference's packer reads from its ``ComputeTile`` / ``Op``
objects (gen_formats_v2.py:2333-2485, :451-523; my_fuse_formats.py:3321-3678)
so that a plan produced here and a plan produced by the reference pack into
identical index arrays.

Template names follow the reference (``get_template_str``,
gen_formats_v2.py:2073-2088):
  "sparse_template_ell"  ELL row-bucket tile (SpMM, CUDA cores)
  "TensorCore_template"  dense 16-row block tile (SpMM, tensor cores)
  "1D_sddmm"             nonzero-chunk tile (SDDMM, CUDA cores)
  "TC_sddmm"             dense 16x16 block tile (SDDMM)
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import scipy.sparse as sp

ELL = "sparse_template_ell"
TC = "TensorCore_template"
ONE_D = "1D_sddmm"
TC_SDDMM = "TC_sddmm"


@dataclass
class OpSpace:
    """The index space of one candidate operator.

    i_perm[p] / k_perm[p]: original row / column at position p
    (``Op.idx_values_list[0][0]`` / ``[2]``).
    """
    op_id: int
    template: str
    i_perm: np.ndarray
    k_perm: np.ndarray
    idx_reordered: tuple = (False, False, False)
    # ELL: folded row -> position row (``Op.hyb_new_rows[0]``), last folded
    # row of every position row, first folded row shorter than the bucket
    hyb_new_rows: Optional[np.ndarray] = None
    hyb_ori_row_ends: Optional[np.ndarray] = None
    hyb_short_begin_row: Optional[int] = None
    # TC: per 16-row block, column order (positions into k_perm)
    # (``Op.k_vals``); a dict {row_block: array} so sparse storage works
    blk_k_vals: Optional[dict] = None
    TC_k_notsorted: bool = False
    # 1D SDDMM: original row / column / output nonzero id per flattened nnz
    ori_row_ids_1d: Optional[np.ndarray] = None
    ori_col_ids_1d: Optional[np.ndarray] = None
    nnz_id_1d: Optional[np.ndarray] = None
    # SDDMM TC: output nonzero id matrix in position space (CSR, data = id+1)
    nnz_id_matrix: Optional[sp.csr_matrix] = None


@dataclass
class Tile:
    op: OpSpace
    tile_sizes: tuple
    tile_pos: tuple
    params: dict
    best_tile_sizes: tuple = None
    best_params: dict = None
    is_atomic: bool = False
    tile_i_rng: Optional[tuple] = None
    tile_k_rng: Optional[tuple] = None
    i_vals: Optional[np.ndarray] = None
    k_vals: Optional[np.ndarray] = None
    # entries covered by this tile (``position_space_when_selected``): a CSR
    # in the op's position space (rows = tile rows) or, for 1D SDDMM, the 0/1
    # vector of still-uncovered nonzeros in the chunk
    covered: object = None
    pred_cost: Optional[float] = None
    nnz_when_selected: Optional[int] = None
    j_num: int = 0
    nnz: int = 0

    @property
    def template(self):
        return self.op.template


def tile_extent(ts):
    """prod(tile_sizes[d][1:]), the reference's per-dimension tile length."""
    out = 1
    for v in ts[1:]:
        out *= int(v)
    return out


@dataclass
class Format:
    """Tiles that share one fused-kernel branch: same template, best tile
    sizes and params (``get_formats_from_selected_tiles``,
    my_fuse_formats.py:121-192)."""
    template: str
    tile_sizes: tuple
    params: dict
    tiles: list = field(default_factory=list)

    @property
    def atomic(self):
        return bool(self.params.get("real_atomic", False))


def _as_tuple(ts):
    if isinstance(ts, (list, tuple)):
        return tuple(_as_tuple(x) for x in ts)
    return ts


def group_formats(tiles, cache_set=("A",)):
    """Group selected tiles into formats keyed by (template, best tile
    sizes, params json) in first-appearance order, adding the scheduling
    flags the reference adds (real_atomic, atomic=False, idx_reordered,
    SMEM_in1)."""
    formats = {}
    for t in tiles:
        params = dict(t.best_params if t.best_params is not None else t.params)
        params["real_atomic"] = bool(t.is_atomic)
        params["atomic"] = False
        params["idx_reordered"] = [bool(x) for x in t.op.idx_reordered]
        params["SMEM_in1"] = "A" in cache_set
        bts = t.best_tile_sizes if t.best_tile_sizes is not None else t.tile_sizes
        key = (t.template, _as_tuple(bts), json.dumps(params))
        if key not in formats:
            formats[key] = Format(t.template, _as_tuple(bts), params)
        formats[key].tiles.append(t)
    return list(formats.values())


@dataclass
class Plan:
    """A complete selected plan for one sparse pattern."""
    op_type: str            # "spmm" | "sddmm"
    shape: tuple            # (M, K) of the sparse matrix
    tiles: list
    max_bucket_size: int = 32
    level_num: int = 1
    meta: dict = field(default_factory=dict)

    def formats(self):
        return group_formats(self.tiles)

    def summary(self):
        out = {}
        for t in self.tiles:
            k = (t.template, bool(t.is_atomic))
            out[k] = out.get(k, 0) + 1
        return out
