"""Rebuild the reference's selected plan stored in a golden fixture as
``stile_gb300.plan`` objects (test helper)."""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from stile_gb300.plan import ONE_D, TC, TC_SDDMM, ELL, OpSpace, Plan, Tile


def _tup(x):
    if isinstance(x, list):
        return tuple(_tup(v) for v in x)
    return x


def plan_from_fixture(meta, arrays):
    ops = {}
    for om in meta["ops"]:
        oid = om["op_id"]
        pre = f"op{oid}_"
        op = OpSpace(op_id=oid, template=om["template"],
                     i_perm=arrays[pre + "i_vals"].astype(np.int64),
                     k_perm=arrays[pre + "k_vals"].astype(np.int64),
                     idx_reordered=tuple(om["idx_reordered"]),
                     TC_k_notsorted=bool(om.get("TC_k_notsorted", False)))
        if om["template"] == ELL:
            op.hyb_new_rows = arrays[pre + "hyb_new_rows"].astype(np.int64)
            op.hyb_ori_row_ends = arrays[pre + "hyb_ori_row_ends"].astype(np.int64)
            op.hyb_short_begin_row = om["hyb_short_begin_row"]
        if om["template"] in (TC, TC_SDDMM):
            rows = arrays[pre + "blk_k_rows"]
            vals = arrays[pre + "blk_k_vals"].astype(np.int64)
            op.blk_k_vals = {int(r): vals[n] for n, r in enumerate(rows)}
        if om["template"] == TC_SDDMM:
            op.nnz_id_matrix = sp.csr_matrix(
                (arrays[pre + "nnzid_data"], arrays[pre + "nnzid_indices"], arrays[pre + "nnzid_indptr"]),
                shape=tuple(om["nnzid_shape"]))
        if om["template"] == ONE_D:
            op.ori_row_ids_1d = arrays[pre + "ori_row_ids_1d"].astype(np.int64)
            op.ori_col_ids_1d = arrays[pre + "ori_col_ids_1d"].astype(np.int64)
            op.nnz_id_1d = arrays[pre + "nnz_id_1d"].astype(np.int64)
        ops[oid] = op
    tiles = []
    for n, tm in enumerate(meta["tiles"]):
        pre = f"t{n}_"
        t = Tile(op=ops[tm["op_id"]], tile_sizes=_tup(tm["tile_sizes"]), tile_pos=tuple(tm["tile_pos"]),
                 params=tm["params"], best_tile_sizes=_tup(tm["best_tile_sizes"]),
                 best_params=tm["params"], is_atomic=tm["is_atomic"],
                 tile_i_rng=None if tm["tile_i_rng"] is None else tuple(tm["tile_i_rng"]),
                 tile_k_rng=None if tm["tile_k_rng"] is None else tuple(tm["tile_k_rng"]),
                 pred_cost=tm["pred_cost"], nnz_when_selected=tm["nnz_when_selected"],
                 j_num=tm["j_num"])
        if pre + "i_vals" in arrays:
            t.i_vals = arrays[pre + "i_vals"].astype(np.int64)
        if pre + "k_vals" in arrays:
            t.k_vals = arrays[pre + "k_vals"].astype(np.int64)
        if pre + "cov_indptr" in arrays:
            t.covered = sp.csr_matrix((arrays[pre + "cov_data"].astype(np.float64),
                                       arrays[pre + "cov_indices"], arrays[pre + "cov_indptr"]),
                                      shape=tuple(tm["cov_shape"]))
        elif pre + "cov_1d" in arrays:
            t.covered = arrays[pre + "cov_1d"]
        tiles.append(t)
    M, _, K = meta["idx_lens"]
    return Plan(op_type=meta["op"], shape=(M, K), tiles=tiles,
                max_bucket_size=meta["max_bucket_size"], meta={"name": meta["name"]})
