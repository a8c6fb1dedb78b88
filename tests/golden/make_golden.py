"""Generate the golden fixtures under tests/golden/ by running the reference
planner and emitter (STile ``MY_sparse``) on small seeded synthetic matrices.

This script only runs where the reference sources are present (it is never
run by the tests, by ``smoke()`` or by the bench).  The reference imports
SparseTIR/TVM, DGL and ``sparsetir_artifact`` at module level although the
planning and packing code never calls them; they are replaced by permissive
stub modules here, exactly like an import-time mock.  ``tvm.nd.array`` is
mapped to ``numpy.asarray`` so ``prepare_inputs_BSPMM`` /
``prepare_inputs_BSDDMM`` return host arrays.

For every case the fixture ``<name>.npz`` holds
  * the input pattern (CSR indptr/indices, shape, feature size N),
  * the reference's selected plan after ``post_process_for_withdraw``,
    serialised tile by tile (template, sizes, position, ranges, i/k values,
    covered CSR, atomicity, predicted cost) plus the per-operator index
    permutations it refers to,
  * the arrays ``prepare_inputs_*`` emitted for that plan, in format order,
  * the format keys (template, best tile sizes, params json).

Usage:  python tests/golden/make_golden.py [--ref PATH] [--only NAME]
"""
from __future__ import annotations

import argparse
import contextlib
import io
import json
import os
import sys
import tempfile
import time
import types

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


# --------------------------------------------------------------------------
# stub modules
# --------------------------------------------------------------------------
class _Perm:
    """Accepts any attribute access, call, subscription or decoration."""

    def __init__(self, name="stub"):
        self._name = name

    def __getattr__(self, item):
        if item.startswith("__") and item.endswith("__"):
            raise AttributeError(item)
        return _Perm(f"{self._name}.{item}")

    def __call__(self, *a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]
        return _Perm(f"{self._name}()")

    def __getitem__(self, item):
        return _Perm(f"{self._name}[]")

    def __iter__(self):
        return iter(())

    def __mro_entries__(self, bases):
        return (object,)


def _stub_module(name, **attrs):
    mod = types.ModuleType(name)
    mod.__path__ = []  # make it a package

    def _ga(item):
        if item.startswith("__") and item.endswith("__"):
            raise AttributeError(item)
        return _Perm(f"{name}.{item}")

    mod.__getattr__ = _ga
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def install_stubs():
    import torch  # noqa: F401  (import before the stubs so nothing shadows it)
    import scipy.sparse  # noqa: F401

    tvm = _stub_module("tvm")
    tvm.nd = types.SimpleNamespace(array=lambda v, device=None: np.asarray(v))
    for sub in ["tvm.testing", "tvm.tir", "tvm.script", "tvm.sparse", "tvm.te",
                "tvm.target", "tvm.contrib", "tvm.runtime", "tvm.ir"]:
        m = _stub_module(sub)
        setattr(tvm, sub.split(".")[1], m)
    sys.modules["tvm.script"].tir = _Perm("T")
    sys.modules["tvm.sparse"].lower_sparse_buffer = _Perm("lsb")
    sys.modules["tvm.sparse"].lower_sparse_iter = _Perm("lsi")
    _stub_module("dgl", DGLError=type("DGLError", (Exception,), {}))
    _stub_module("sparsetir_artifact", profile_pytorch_ms=_Perm("p"), profile_tvm_ms=_Perm("p"))
    _stub_module("ogb")
    _stub_module("ogb.nodeproppred")


def import_reference(ref_root):
    """Import the reference modules (their MLP weights load by relative path
    at import, so cwd must be MY_sparse during the import)."""
    install_stubs()
    src = os.path.join(ref_root, "MY_sparse")
    sys.path.insert(0, src)
    old = os.getcwd()
    os.chdir(src)
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            import gen_formats_v2 as G
            import my_search_formats as S
            import my_branch_and_bound as BB
            import my_fuse_formats as F
            import my_cost_model as CM
    finally:
        os.chdir(old)
    return G, S, BB, F, CM


# --------------------------------------------------------------------------
# cases
# --------------------------------------------------------------------------
def _cases():
    from stile_gb300 import synthetic as syn

    def pl(m, k, min_len, max_len, seed):
        return syn.power_law_rows(m, k, exponent=2.1, min_len=min_len, max_len=max_len,
                                  seed=seed, values="ones")

    return {
        # power-law rows (scaled-down plain SpMM workload)
        "spmm_powerlaw_512": dict(op="spmm", A=lambda: pl(512, 512, 1, 128, 11), N=64,
                                  only_TC=False, only_ELL=False),
        "spmm_powerlaw_1024_min4": dict(op="spmm", A=lambda: pl(1024, 1024, 4, 256, 12), N=64,
                                        only_TC=False, only_ELL=False),
        "spmm_powerlaw_512_ell": dict(op="spmm", A=lambda: pl(512, 512, 1, 128, 13), N=32,
                                      only_TC=False, only_ELL=True),
        # the plain SpMM workload at full size (4096^2, exponent 2.1, lengths 1..1024)
        "spmm_powerlaw_4096": dict(op="spmm", A=lambda: pl(4096, 4096, 1, 1024, 0), N=64,
                                   only_TC=False, only_ELL=False),
        "spmm_powerlaw_4096_min10": dict(op="spmm", A=lambda: pl(4096, 4096, 10, 1024, 0), N=64,
                                         only_TC=False, only_ELL=False),
        # graph with planted 16x16 communities (scaled-down hybrid workload)
        "spmm_community_1024": dict(op="spmm",
                                    A=lambda: syn.community_graph(n=1024, target_nnz=12000, seed=3,
                                                                  values="ones", max_deg=256),
                                    N=128, only_TC=False, only_ELL=False),
        "spmm_community_2048": dict(op="spmm",
                                    A=lambda: syn.community_graph(n=2048, target_nnz=30000, seed=4,
                                                                  values="ones", max_deg=512),
                                    N=128, only_TC=False, only_ELL=False),
        "spmm_community_8192": dict(op="spmm",
                                    A=lambda: syn.community_graph(n=8192, target_nnz=60000, seed=9,
                                                                  values="ones", max_deg=1024),
                                    N=128, only_TC=False, only_ELL=False),
        # dense blocks next to hub rows (atomic TC tiles, then withdraw)
        "spmm_hubblocks_4096": dict(op="spmm", A=lambda: _hub_blocks(4096, 4, 60, 1500), N=64,
                                    only_TC=False, only_ELL=False),
        # power-law rows + dense blocks (atomic ELL tiles next to TC tiles)
        "spmm_mixed_2048": dict(op="spmm", A=lambda: _mixed_blocks(2048, 1, 40, 8, 256), N=64,
                                only_TC=False, only_ELL=False),
        # block + unstructured pruned weight (scaled-down)
        "spmm_pruned_256x192": dict(op="spmm",
                                    A=lambda: _ones(syn.pruned_weight(256, 192, seed=5)),
                                    N=64, only_TC=False, only_ELL=False),
        "spmm_pruned_256x192_tc": dict(op="spmm",
                                       A=lambda: _ones(syn.pruned_weight(256, 192, seed=6)),
                                       N=64, only_TC=True, only_ELL=False),
        # block-structured weights with the tensor-core columns kept in their
        # order (TC_k_notsorted): tiles are 16x16 blocks on the column grid
        "spmm_blockpruned_768x512_knots": dict(
            op="spmm", A=lambda: _ones(syn.pruned_weight(768, 512, sparsity=0.95, block_frac=0.8, seed=21)),
            N=64, only_TC=False, only_ELL=False, TC_k_notsorted=True),
        "spmm_blockpruned_768x512_knots_tc": dict(
            op="spmm", A=lambda: _ones(syn.pruned_weight(768, 512, sparsity=0.95, block_frac=0.8, seed=22)),
            N=64, only_TC=True, only_ELL=False, TC_k_notsorted=True),
        # SDDMM mask: power-law rows + dense 32x16 blocks
        "sddmm_mask_1024": dict(op="sddmm",
                                A=lambda: syn.sddmm_mask(n=1024, target_nnz=16000, seed=7, max_len=256),
                                N=64, only_TC=False, only_ELL=False),
        "sddmm_mask_2048": dict(op="sddmm",
                                A=lambda: syn.sddmm_mask(n=2048, target_nnz=40000, seed=8, max_len=512),
                                N=32, only_TC=False, only_ELL=False),
        # the ablation switches: one level of operators (max_level_num 1) and
        # whole-row tensor-core tiles costed without withdraw
        "spmm_community_1024_single_level": dict(
            op="spmm", A=lambda: syn.community_graph(n=1024, target_nnz=12000, seed=3, values="ones", max_deg=256),
            N=128, only_TC=False, only_ELL=False, single_level=True),
        "spmm_hubblocks_4096_no_withdraw": dict(op="spmm", A=lambda: _hub_blocks(4096, 4, 60, 1500), N=64,
                                                only_TC=False, only_ELL=False, no_withdraw=True),
        "sddmm_mask_1024_single_level": dict(
            op="sddmm", A=lambda: syn.sddmm_mask(n=1024, target_nnz=16000, seed=7, max_len=256),
            N=64, only_TC=False, only_ELL=False, single_level=True),
        # the local-search ablation (my_run_localsearch.py: cost window 1e-6)
        "spmm_mixed_2048_window0": dict(op="spmm", A=lambda: _mixed_blocks(2048, 1, 40, 8, 256), N=64,
                                        only_TC=False, only_ELL=False, max_avg_cost_diff=1e-6),
        "sddmm_mask_1024_1d": dict(op="sddmm",
                                   A=lambda: syn.sddmm_mask(n=1024, target_nnz=16000, seed=7, max_len=256),
                                   N=64, only_TC=False, only_ELL=True),
        # tensor-core columns: non-empty first in column order
        # (reorder_k_by_nnz=False)
        "spmm_community_2048_kfirst": dict(op="spmm",
                                           A=lambda: syn.community_graph(n=2048, target_nnz=30000, seed=4,
                                                                         values="ones", max_deg=512),
                                           N=128, only_TC=False, only_ELL=False, reorder_k_by_nnz=False),
        "sddmm_mask_1024_tc": dict(op="sddmm",
                                   A=lambda: syn.sddmm_mask(n=1024, target_nnz=16000, seed=7, max_len=256),
                                   N=64, only_TC=True, only_ELL=False),
        "sddmm_mask_1024_knots_tc": dict(op="sddmm",
                                         A=lambda: syn.sddmm_mask(n=1024, target_nnz=16000, seed=7, max_len=256),
                                         N=64, only_TC=True, only_ELL=False, TC_k_notsorted=True),
        "sddmm_mask_1024_knots": dict(op="sddmm",
                                      A=lambda: syn.sddmm_mask(n=1024, target_nnz=16000, seed=7, max_len=256),
                                      N=64, only_TC=False, only_ELL=False, TC_k_notsorted=True),
    }


def _hub_blocks(n, seed, nblk, hub_len, bw=64):
    """Power-law rows plus dense 16 x bw blocks, each sharing its 16-row
    window with one long (hub) row: atomic tensor-core tiles are selected
    first and later withdrawn in favour of whole-row tiles."""
    from stile_gb300 import synthetic as syn
    rng = np.random.default_rng(seed)
    A = syn.power_law_rows(n, n, min_len=2, max_len=64, seed=seed, values="ones").tolil()
    for _ in range(nblk):
        r = rng.integers(0, n // 16) * 16
        c = rng.integers(0, n - bw)
        A[r:r + 16, c:c + bw] = 1
        A[r + rng.integers(0, 16), rng.choice(n, size=hub_len, replace=False)] = 1
    return _ones(sp.csr_matrix(A))


def _mixed_blocks(n, seed, nblk, min_len, max_len, bw=64):
    """Power-law rows plus dense 16 x bw blocks anywhere."""
    from stile_gb300 import synthetic as syn
    rng = np.random.default_rng(seed)
    A = syn.power_law_rows(n, n, min_len=min_len, max_len=max_len, seed=seed, values="ones").tolil()
    for _ in range(nblk):
        r = rng.integers(0, n // 16) * 16
        c = rng.integers(0, n - bw)
        A[r:r + 16, c:c + bw] = 1
    return _ones(sp.csr_matrix(A))


def _ones(A):
    A = A.tocsr().copy()
    A.data[:] = 1.0
    return A


# --------------------------------------------------------------------------
# running the reference
# --------------------------------------------------------------------------
def build_ref_op(G, op_type, A, N):
    """Mirror of the reference's graph loader (gen_formats_v2.py:2709-2789):
    shape padded to multiples of 128 (SpMM) / 128x160 (SDDMM), values 1."""
    import math
    M0, K0 = A.shape
    if op_type == "spmm":
        idx_lens = [math.ceil(M0 / 128) * 128, N, math.ceil(K0 / 128) * 128]
    else:
        idx_lens = [math.ceil(M0 / 128) * 128, N, math.ceil(K0 / 160) * 160]
    indptr = np.concatenate([A.indptr, np.full(idx_lens[0] - M0, A.indptr[-1])])
    A_csr = sp.csr_matrix((np.full(A.nnz, 1, dtype="float32"), A.indices, indptr),
                          shape=(idx_lens[0], idx_lens[2]))
    A_csr.sum_duplicates()
    A_csr = sp.csr_matrix((np.full(len(A_csr.data), 1, dtype="float32"), A_csr.indices, A_csr.indptr),
                          shape=(idx_lens[0], idx_lens[2]))
    rng = np.random.default_rng(seed=0)
    if op_type == "spmm":
        Bs = [rng.random((idx_lens[2], N)).astype("float32")]
    else:
        Bs = [rng.random((idx_lens[0], N)).astype("float32"),
              rng.random((idx_lens[2], N)).astype("float32")]
    inps = [A_csr] + [G.DenseTensor(B) for B in Bs]
    with contextlib.redirect_stdout(io.StringIO()):
        op = G.Op(op_type, [0, 1], [2], idx_lens, None, inps, [A_csr.tocsc()])
    return op


def run_reference(mods, case):
    G, S, BB, F, CM = mods
    op_type = case["op"]
    os.environ["op_type"] = op_type
    single = bool(case.get("single_level", False))
    os.environ["single_level"] = str(single)
    knots = bool(case.get("TC_k_notsorted", False))
    os.environ["TC_k_notsorted"] = str(knots)
    os.environ["no_withdraw"] = str(bool(case.get("no_withdraw", False)))
    os.environ["REMAP"] = "False"
    os.environ.pop("TC_tile_sizes", None)
    os.environ["other_cost_model"] = "analytic"
    A = case["A"]()
    op = build_ref_op(G, op_type, A, case["N"])
    # driver constants of SPMM/SPMMbench_our_method.py:187-222 and
    # SDDMM/SDDMMbench_our_method.py (dsize 16, cache_set ['A'], fp16)
    dsize = 16
    cache_set = ["A"]
    kernel_tile_size_options = ([1], [1], [1])
    max_avg_cost_diff = case.get("max_avg_cost_diff", 0.2)
    only_TC, only_ELL = case["only_TC"], case["only_ELL"]
    if only_ELL:
        max_avg_cost_diff = float("inf")
    mbs = S.estimate_max_bucket_size(op)
    if op_type == "sddmm":
        mbs = 32
    t0 = time.time()
    log = io.StringIO()
    with contextlib.redirect_stdout(log):
        res = S.greedy_search_use_cost_model_lower_bound(
            op, dsize, {"summarize_nnz_iter_space": (True, True)}, mbs, cache_set,
            kernel_tile_size_options, only_TC, only_ELL, 1, knots,
            reorder_k_by_nnz=case.get("reorder_k_by_nnz", True), max_level_num=1 if single else float("inf"),
            max_avg_cost_diff=max_avg_cost_diff, use_faster_tuner=True,
            log_file="log.py", cuda_i=0, dtype="float16", dtype_str='"float16"',
            zerotype="T.float16(0)")
        selected, TC_row_tile_dict, TC_row_costs, reverse_idx, level_num = res
        pre_withdraw = list(selected)
        selected = BB.post_process_for_withdraw(op, selected, TC_row_tile_dict, TC_row_costs, reverse_idx)
    t_search = time.time() - t0
    return op, A, mbs, pre_withdraw, selected, TC_row_costs, reverse_idx, t_search


def _template(G, tile):
    return G.get_template_str(tile.op)


def serialise(mods, case_name, case, op, A, mbs, selected, TC_row_costs, reverse_idx, t_search):
    """Flatten the reference plan + emitted arrays into a dict of arrays."""
    G, S, BB, F, CM = mods
    out = {}
    meta = {"name": case_name, "op": case["op"], "N": case["N"], "idx_lens": list(map(int, op.idx_lens)),
            "orig_shape": list(map(int, A.shape)), "max_bucket_size": int(mbs),
            "only_TC": case["only_TC"], "only_ELL": case["only_ELL"],
            "TC_k_notsorted": bool(case.get("TC_k_notsorted", False)),
            "single_level": bool(case.get("single_level", False)),
            "no_withdraw": bool(case.get("no_withdraw", False)),
            "max_avg_cost_diff": case.get("max_avg_cost_diff", 0.2),
            "reorder_k_by_nnz": case.get("reorder_k_by_nnz", True), "search_s": t_search}
    Ar = op.inps[0]
    out["A_indptr"] = Ar.indptr.astype(np.int32)
    out["A_indices"] = Ar.indices.astype(np.int32)
    out["TC_row_costs"] = np.asarray(TC_row_costs, dtype=np.float64)
    out["reverse_idx_TC_op_row"] = np.asarray(reverse_idx, dtype=np.int32)

    # operators referenced by tiles
    ops = {}
    for t in selected:
        o = t.op
        if o.op_id in ops:
            continue
        ops[o.op_id] = o
    op_meta = []
    for oid, o in ops.items():
        tpl = G.get_template_str(o)
        pre = f"op{oid}_"
        out[pre + "i_vals"] = np.asarray(o.idx_values_list[0][0], dtype=np.int32)
        out[pre + "k_vals"] = np.asarray(o.idx_values_list[0][2], dtype=np.int32)
        om = {"op_id": int(oid), "template": tpl, "idx_reordered": [bool(x) for x in o.idx_reordered[0]],
              "TC_k_notsorted": bool(getattr(o, "TC_k_notsorted", False))}
        if tpl == "sparse_template_ell":
            out[pre + "hyb_new_rows"] = np.asarray(o.hyb_new_rows[0], dtype=np.int32)
            out[pre + "hyb_ori_row_ends"] = np.asarray(o.hyb_ori_row_ends, dtype=np.int32)
            om["hyb_short_begin_row"] = int(o.hyb_short_begin_row)
            ps = o.position_space[0]
            out[pre + "ps_indptr"] = ps.indptr.astype(np.int32)
            out[pre + "ps_indices"] = ps.indices.astype(np.int32)
        if tpl in ("TensorCore_template", "TC_sddmm"):
            kv = o.k_vals
            used = sorted({int(t.tile_pos[0]) for t in selected if t.op.op_id == oid})
            out[pre + "blk_k_rows"] = np.asarray(used, dtype=np.int32)
            out[pre + "blk_k_vals"] = np.stack([np.asarray(kv[r], dtype=np.int32) for r in used])
        if tpl == "TC_sddmm":
            nm = o.nnz_id_matrix.tocsr()
            out[pre + "nnzid_indptr"] = nm.indptr.astype(np.int32)
            out[pre + "nnzid_indices"] = nm.indices.astype(np.int32)
            out[pre + "nnzid_data"] = nm.data.astype(np.int32)
            om["nnzid_shape"] = [int(nm.shape[0]), int(nm.shape[1])]
        if tpl == "1D_sddmm":
            out[pre + "ori_row_ids_1d"] = np.asarray(o.ori_row_ids_1d, dtype=np.int32)
            out[pre + "ori_col_ids_1d"] = np.asarray(o.ori_col_ids_1d, dtype=np.int32)
            out[pre + "nnz_id_1d"] = np.asarray(o.nnz_id_matrix, dtype=np.int32)
        op_meta.append(om)
    meta["ops"] = op_meta

    tiles_meta = []
    for n, t in enumerate(selected):
        tpl = _template(G, t)
        tm = {"op_id": int(t.op.op_id), "template": tpl,
              "tile_sizes": json.loads(json.dumps(t.tile_sizes)),
              "best_tile_sizes": json.loads(json.dumps(t.best_tile_sizes)),
              "tile_pos": [int(x) for x in t.tile_pos] if not isinstance(t.tile_pos, int) else [int(t.tile_pos)],
              "params": t.best_params, "is_atomic": bool(t.is_atomic_tile),
              "pred_cost": float(t.pred_cost) if t.pred_cost is not None else None,
              "nnz_when_selected": int(t.nnz_when_selected) if t.nnz_when_selected is not None else None,
              "j_num": int(t.j_num),
              "tile_i_rng": None if t.tile_i_rng is None else [int(x) for x in t.tile_i_rng],
              "tile_k_rng": None if t.tile_k_rng is None else [int(x) for x in t.tile_k_rng]}
        pre = f"t{n}_"
        if t.i_vals is not None:
            out[pre + "i_vals"] = np.asarray(t.i_vals, dtype=np.int32)
        if t.k_vals is not None:
            out[pre + "k_vals"] = np.asarray(t.k_vals, dtype=np.int32)
        ps = t.position_space_when_selected
        if ps is not None:
            if sp.issparse(ps):
                ps = ps.tocsr()
                out[pre + "cov_indptr"] = ps.indptr.astype(np.int32)
                out[pre + "cov_indices"] = ps.indices.astype(np.int32)
                out[pre + "cov_data"] = np.asarray(ps.data, dtype=np.float32)
                tm["cov_shape"] = [int(ps.shape[0]), int(ps.shape[1])]
            else:
                out[pre + "cov_1d"] = np.asarray(ps, dtype=np.float32)
        tiles_meta.append(tm)
    meta["tiles"] = tiles_meta

    # emitted arrays
    with contextlib.redirect_stdout(io.StringIO()):
        formats = F.get_formats_from_selected_tiles(selected, ["A"], 16)
    fmt_keys = []
    for key, tiles in formats.items():
        fmt_keys.append({"template": key[0], "tile_sizes": json.loads(json.dumps(key[1])),
                         "params": key[2], "n_tiles": len(tiles),
                         "tile_ids": [selected.index(t) for t in tiles]})
    meta["formats"] = fmt_keys
    N = case["N"]
    M = op.idx_lens[0]
    if case["op"] == "spmm":
        has_tc = any(k[0] == "TensorCore_template" for k in formats)
        max_i = M + 1
        max_j = N
        if has_tc:
            max_i = max(max_i, int(np.ceil(M / 16) * 16))
            max_j = max(max_j, int(F.get_padded_j_TC(N, 16)))
        out_shape = (max_i, max_j)
        with contextlib.redirect_stdout(io.StringIO()):
            args, _ = F.prepare_inputs_BSPMM(op, "spmm", 1, formats, out_shape, "float32", None)
        meta["out_shape"] = list(out_shape)
    else:
        with contextlib.redirect_stdout(io.StringIO()):
            args, c_idx = F.prepare_inputs_BSDDMM(op, "sddmm", 1, formats, None, "float32", None)
        meta["c_indices"] = [list(map(int, c)) for c in c_idx]
    # the leading dense operands (b, c for SpMM; a, b, c, a, b for SDDMM) are
    # not plan data: keep their shapes only
    n_dense = 2 if case["op"] == "spmm" else 5
    meta["dense_arg_shapes"] = [list(np.asarray(a).shape) for a in args[:n_dense]]
    for n, a in enumerate(args):
        if n < n_dense:
            continue
        a = np.asarray(a)
        if a.dtype == object:
            # k-block positions of TC_k_notsorted tiles (integral Fractions)
            a = a.astype(np.int64)
        if a.dtype.kind == "f" and a.size and np.all(a == 0):
            meta.setdefault("zero_args", {})[str(n)] = list(a.shape)
            continue
        out[f"arg{n}"] = a.astype(np.int32) if a.dtype.kind in "iu" else a.astype(np.float32)
    meta["n_args"] = len(args)
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the STile project checkout")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    mods = import_reference(args.ref)
    work = tempfile.mkdtemp(prefix="stile_golden_")
    os.chdir(work)  # the reference writes sidecar JSON files into cwd
    for name, case in _cases().items():
        if args.only and name != args.only:
            continue
        t0 = time.time()
        op, A, mbs, pre, selected, costs, rev, t_search = run_reference(mods, case)
        blob = serialise(mods, name, case, op, A, mbs, selected, costs, rev, t_search)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **blob)
        n_tpl = {}
        for t in selected:
            k = mods[0].get_template_str(t.op)
            n_tpl[k] = n_tpl.get(k, 0) + 1
        print(f"{name}: nnz={A.nnz} tiles={n_tpl} search={t_search:.1f}s "
              f"size={os.path.getsize(path)/1024:.0f}KB total={time.time()-t0:.1f}s", flush=True)


if __name__ == "__main__":
    main()
