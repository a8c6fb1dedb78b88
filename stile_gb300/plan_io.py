"""On-disk plan format and a plan cache keyed by sparsity pattern.

The format search is the expensive part of planning: seconds for a graph of a
few hundred thousand nonzeros and minutes at tens of millions (the reference
spends minutes to hours in its greedy / branch-and-bound search,
my_search_formats.py:263, and keeps its tuning results in memory only,
``tuning_hub`` at my_search_formats.py:294).  A plan depends only on the
pattern, the dense width and the search settings, so it is saved once and
reused by later runs, by the backward's transposed operator and by other
processes.

File layout: one uncompressed ``.npz`` (read with ``allow_pickle=False``) that
holds a UTF-8 JSON header in ``header`` and plain integer / float arrays
(64-bit integers stored as int32 where they fit):

* header: format version, op type, shape, bucket size, level count, plan
  meta, the pattern key of the matrix the plan was made for, one record per
  candidate operator (scalar fields, which arrays it has) and a table of the
  distinct (tile sizes, params, best tile sizes, best params) combinations;
* per operator ``s<j>.<field>``: its index arrays (identity permutations are
  stored as their length only), and for tensor-core operators the column
  order of every 16-row block at the positions its tiles read
  (``s<j>.kv_block / kv_ptr / kv_pos / kv_val``), not the whole order;
* per tile, in plan order: operator, descriptor, position (numerator and
  denominator, so fractional k positions survive), row / column ranges,
  atomic flag, predicted cost, counts, and the concatenated ``i_vals``,
  ``k_vals``, covered-entry CSRs (or 0/1 vectors for 1D SDDMM chunks) and
  covered nonzero ids with offset arrays.

A loaded plan emits and packs into the same arrays, bit for bit, as the plan
that was saved.
"""
from __future__ import annotations

import hashlib
import json
import os
import tempfile
import zipfile
from fractions import Fraction

import numpy as np
import scipy.sparse as sp

from .plan import OpSpace, Plan, Tile

FORMAT_VERSION = 1

_SPACE_ARRAYS = ("i_perm", "k_perm", "hyb_new_rows", "hyb_ori_row_ends", "ori_row_ids_1d", "ori_col_ids_1d",
                 "nnz_id_1d")


def pattern_key(A) -> str:
    """Hash of a sparsity pattern (shape + CSR structure)."""
    A = sp.csr_matrix(A)
    A.sort_indices()
    h = hashlib.sha1()
    h.update(np.asarray(A.shape, dtype=np.int64).tobytes())
    h.update(A.indptr.astype(np.int64).tobytes())
    h.update(A.indices.astype(np.int64).tobytes())
    return h.hexdigest()


# ---------------------------------------------------------------------------
# tagged JSON for tile sizes / params (tuples, lists, fractions, None)
# ---------------------------------------------------------------------------
def _enc(x):
    if isinstance(x, tuple):
        return {"t": [_enc(v) for v in x]}
    if isinstance(x, list):
        return [_enc(v) for v in x]
    if isinstance(x, dict):
        return {"d": [[str(k), _enc(v)] for k, v in x.items()]}
    if isinstance(x, Fraction):
        return {"q": [x.numerator, x.denominator]}
    if isinstance(x, (bool, np.bool_)):
        return bool(x)
    if isinstance(x, (int, np.integer)):
        return int(x)
    if isinstance(x, (float, np.floating)):
        return float(x)
    if x is None or isinstance(x, str):
        return x
    raise TypeError(f"cannot store {type(x).__name__} in a plan file")


def _dec(x):
    if isinstance(x, list):
        return [_dec(v) for v in x]
    if isinstance(x, dict):
        if "t" in x:
            return tuple(_dec(v) for v in x["t"])
        if "d" in x:
            return {k: _dec(v) for k, v in x["d"]}
        if "q" in x:
            return Fraction(*x["q"])
    return x


# ---------------------------------------------------------------------------
# stored column orders of tensor-core blocks
# ---------------------------------------------------------------------------
class StoredBlockOrder:
    """Column order of one 16-row block, known at the positions the plan's
    tiles read (sorted ``pos``, values ``val``); any other position is an
    error, never a guess."""

    def __init__(self, pos, val, length):
        self.pos, self.val, self.length = pos, val, int(length)

    def __len__(self):
        return self.length

    def __getitem__(self, idx):
        if isinstance(idx, slice):
            idx = np.arange(*idx.indices(self.length))
        scalar = np.ndim(idx) == 0
        q = np.atleast_1d(np.asarray(idx, dtype=np.int64))
        q = np.where(q < 0, q + self.length, q)
        j = np.searchsorted(self.pos, q)
        if len(q) and (np.any(j >= len(self.pos)) or np.any(self.pos[np.minimum(j, len(self.pos) - 1)] != q)):
            raise KeyError("block column order was not stored at the requested positions")
        out = self.val[j]
        return out[0] if scalar else out


class StoredKvals(dict):
    """``blk_k_vals`` of a loaded plan: {row block: StoredBlockOrder}."""


def _kvals_positions(tile):
    """Positions of the block's column order that emitting ``tile`` reads."""
    if tile.tile_k_rng is not None:
        k0, k1 = tile.tile_k_rng
        return np.arange(int(k0), int(k1) + 1, dtype=np.int64)
    return np.asarray(tile.k_vals, dtype=np.int64)


# ---------------------------------------------------------------------------
# save
# ---------------------------------------------------------------------------
def _cat(parts, dtype):
    return np.concatenate(parts).astype(dtype) if parts else np.zeros(0, dtype)


def _ptr(lengths):
    return np.concatenate([[0], np.cumsum(np.asarray(lengths, dtype=np.int64))]).astype(np.int64)


def plan_arrays(plan: Plan, pattern: str | None = None):
    """(header dict, {name: array}) for ``plan``."""
    arrays = {}
    spaces, space_of = [], {}
    for t in plan.tiles:
        if id(t.op) not in space_of:
            space_of[id(t.op)] = len(spaces)
            spaces.append(t.op)

    # column orders read by the tiles, per operator and block
    kv_needed = [dict() for _ in spaces]
    for t in plan.tiles:
        op = t.op
        if op.blk_k_vals is None or t.template not in ("TensorCore_template", "TC_sddmm"):
            continue
        b = int(t.tile_pos[0])
        kv_needed[space_of[id(op)]].setdefault(b, []).append(_kvals_positions(t))

    space_recs = []
    for j, op in enumerate(spaces):
        rec = {"op_id": int(op.op_id), "template": op.template, "idx_reordered": [bool(x) for x in op.idx_reordered],
               "hyb_short_begin_row": None if op.hyb_short_begin_row is None else int(op.hyb_short_begin_row),
               "TC_k_notsorted": bool(op.TC_k_notsorted), "arrays": {}, "kvals": op.blk_k_vals is not None,
               "nnz_id_matrix": None}
        for name in _SPACE_ARRAYS:
            a = getattr(op, name)
            if a is None:
                continue
            a = np.asarray(a)
            if a.ndim == 1 and np.issubdtype(a.dtype, np.integer) and np.array_equal(a, np.arange(len(a))):
                rec["arrays"][name] = {"arange": int(len(a)), "dtype": str(a.dtype)}
            else:
                rec["arrays"][name] = {"dtype": str(a.dtype)}
                arrays[f"s{j}.{name}"] = a
        if op.blk_k_vals is not None:
            blocks = sorted(kv_needed[j])
            pos_l, val_l, lens, blen = [], [], [], []
            for b in blocks:
                pos = np.unique(np.concatenate(kv_needed[j][b]))
                order = op.blk_k_vals[b]
                blen.append(len(order))
                pos_l.append(pos)
                val_l.append(np.asarray(order[pos], dtype=np.int64).reshape(-1))
                lens.append(len(pos))
            arrays[f"s{j}.kv_block"] = np.asarray(blocks, dtype=np.int64)
            arrays[f"s{j}.kv_ptr"] = _ptr(lens)
            arrays[f"s{j}.kv_blen"] = np.asarray(blen, dtype=np.int64)
            arrays[f"s{j}.kv_pos"] = _cat(pos_l, np.int64)
            arrays[f"s{j}.kv_val"] = _cat(val_l, np.int64)
        if op.nnz_id_matrix is not None:
            m = sp.csr_matrix(op.nnz_id_matrix)
            rec["nnz_id_matrix"] = {"shape": [int(m.shape[0]), int(m.shape[1])], "dtype": str(m.data.dtype),
                                    "sorted": bool(m.has_sorted_indices)}
            arrays[f"s{j}.nzm_indptr"] = m.indptr.astype(np.int64)
            arrays[f"s{j}.nzm_indices"] = m.indices.astype(np.int64)
            arrays[f"s{j}.nzm_data"] = m.data
        space_recs.append(rec)

    # per-tile records
    n = len(plan.tiles)
    desc_idx, desc_tab = np.zeros(n, np.int64), {}
    pos_num = np.zeros((n, 3), np.int64)
    pos_den = np.zeros((n, 3), np.int64)
    pos_len = np.zeros(n, np.int64)
    i_rng = np.full((n, 2), -1, np.int64)
    k_rng = np.full((n, 2), -1, np.int64)
    rng_set = np.zeros((n, 2), np.int8)
    flags = np.zeros((n, 4), np.int64)      # space, is_atomic, j_num, nnz
    nnz_sel = np.full(n, -1, np.int64)
    pred = np.full(n, np.nan)
    iv_l, iv_len, kv_l, kv_len = [], [], [], []
    cov_kind = np.zeros(n, np.int8)          # 0 none, 1 CSR, 2 vector
    cov_shape = np.zeros((n, 2), np.int64)
    ci_l, cj_l, cd_l, crow_len, cnnz_len = [], [], [], [], []
    vec_l, vec_len = [], []
    ids_l, ids_len, has_ids = [], [], np.zeros(n, np.int8)
    for i, t in enumerate(plan.tiles):
        d = json.dumps([_enc(t.tile_sizes), _enc(t.params), _enc(t.best_tile_sizes), _enc(t.best_params)])
        desc_idx[i] = desc_tab.setdefault(d, len(desc_tab))
        pos = tuple(t.tile_pos)
        if len(pos) > 3:
            raise ValueError("tile positions have at most three coordinates")
        pos_len[i] = len(pos)
        for c, v in enumerate(pos):
            if isinstance(v, Fraction):
                pos_num[i, c], pos_den[i, c] = v.numerator, v.denominator
            else:
                pos_num[i, c] = int(v)
        for c, r in enumerate((t.tile_i_rng, t.tile_k_rng)):
            if r is not None:
                (i_rng if c == 0 else k_rng)[i] = [int(r[0]), int(r[1])]
                rng_set[i, c] = 1
        flags[i] = [space_of[id(t.op)], int(bool(t.is_atomic)), int(t.j_num), int(t.nnz)]
        if t.nnz_when_selected is not None:
            nnz_sel[i] = int(t.nnz_when_selected)
        if t.pred_cost is not None:
            pred[i] = float(t.pred_cost)
        iv = np.zeros(0, np.int64) if t.i_vals is None else np.asarray(t.i_vals, np.int64)
        kv = np.zeros(0, np.int64) if t.k_vals is None else np.asarray(t.k_vals, np.int64)
        iv_l.append(iv); iv_len.append(len(iv) if t.i_vals is not None else -1)
        kv_l.append(kv); kv_len.append(len(kv) if t.k_vals is not None else -1)
        cov = t.covered
        if cov is None:
            crow_len.append(0); cnnz_len.append(0); vec_len.append(0)
        elif sp.issparse(cov):
            m = sp.csr_matrix(cov)
            cov_kind[i] = 1
            cov_shape[i] = m.shape
            ci_l.append(m.indptr.astype(np.int64)); crow_len.append(len(m.indptr))
            cj_l.append(m.indices.astype(np.int64)); cd_l.append(np.asarray(m.data, np.float64))
            cnnz_len.append(m.nnz); vec_len.append(0)
        else:
            v = np.asarray(cov, np.float64).reshape(-1)
            cov_kind[i] = 2
            cov_shape[i] = [len(v), 0]
            vec_l.append(v); vec_len.append(len(v))
            crow_len.append(0); cnnz_len.append(0)
        ids = getattr(t, "cov_ids", None)
        if ids is not None:
            has_ids[i] = 1
            ids_l.append(np.asarray(ids, np.int64)); ids_len.append(len(ids))
        else:
            ids_len.append(0)
    cov_data = _cat(cd_l, np.float64)
    ones = bool(np.all(cov_data == 1.0))
    arrays.update({
        "t.desc": desc_idx, "t.pos_num": pos_num, "t.pos_den": pos_den, "t.pos_len": pos_len,
        "t.i_rng": i_rng, "t.k_rng": k_rng, "t.rng_set": rng_set, "t.flags": flags, "t.nnz_sel": nnz_sel,
        "t.pred": pred,
        "t.iv_len": np.asarray(iv_len, np.int64), "t.iv": _cat(iv_l, np.int64),
        "t.kv_len": np.asarray(kv_len, np.int64), "t.kv": _cat(kv_l, np.int64),
        "t.cov_kind": cov_kind, "t.cov_shape": cov_shape,
        "t.cov_row_len": np.asarray(crow_len, np.int64), "t.cov_indptr": _cat(ci_l, np.int64),
        "t.cov_nnz_len": np.asarray(cnnz_len, np.int64), "t.cov_indices": _cat(cj_l, np.int64),
        "t.cov_vec_len": np.asarray(vec_len, np.int64), "t.cov_vec": _cat(vec_l, np.float64),
        "t.has_ids": has_ids, "t.ids_len": np.asarray(ids_len, np.int64), "t.ids": _cat(ids_l, np.int64),
    })
    if not ones:
        arrays["t.cov_data"] = cov_data
    header = {"format": "stile_gb300.plan", "version": FORMAT_VERSION, "op_type": plan.op_type,
              "shape": [int(x) for x in plan.shape], "max_bucket_size": int(plan.max_bucket_size),
              "level_num": int(plan.level_num), "meta": plan.meta, "pattern": pattern, "spaces": space_recs,
              "descriptors": sorted(desc_tab, key=desc_tab.get), "n_tiles": n, "cov_data_ones": ones}
    return header, arrays


def _narrow(a):
    """64-bit integer arrays whose values fit are stored as int32 (all
    integer arrays are read back as int64, then cast to the dtype the
    header records where it records one)."""
    if a.dtype == np.int64 and a.size and a.min() >= -(1 << 31) and a.max() < (1 << 31):
        return a.astype(np.int32)
    return a


def _write(path, header, arrays):
    arrays = {k: _narrow(np.asarray(v)) for k, v in arrays.items()}
    arrays["header"] = np.frombuffer(json.dumps(header).encode("utf-8"), dtype=np.uint8)
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d, suffix=".npz.tmp")
    try:
        with os.fdopen(fd, "wb") as f:
            np.savez(f, **arrays)
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


def save_plan(plan: Plan, path: str, A=None, pattern: str | None = None):
    """Write ``plan`` to ``path`` (an ``.npz``).  With the matrix ``A`` (or
    its ``pattern`` key) the file records the pattern key, which
    ``load_plan`` checks.  The file appears atomically (written beside the
    target, then renamed)."""
    if pattern is None and A is not None:
        pattern = pattern_key(A)
    _write(path, *plan_arrays(plan, pattern))


# ---------------------------------------------------------------------------
# load
# ---------------------------------------------------------------------------
def _split(flat, lengths):
    """Pieces of ``flat`` of the given lengths (-1: None)."""
    out, o = [], 0
    for n in lengths:
        n = int(n)
        if n < 0:
            out.append(None)
            continue
        out.append(flat[o:o + n])
        o += n
    if o != len(flat):
        raise ValueError("plan file: array lengths do not add up")
    return out


def load_plan(path: str, A=None, pattern: str | None = None) -> Plan:
    """Read a plan written by ``save_plan``.  With ``A`` (or its
    ``pattern`` key), the file's pattern key must match (ValueError
    otherwise)."""
    with np.load(path, allow_pickle=False) as z:
        arrays = {k: (z[k].astype(np.int64) if z[k].dtype == np.int32 else z[k]) for k in z.files}
    header = json.loads(arrays.pop("header").tobytes().decode("utf-8"))
    if header.get("format") != "stile_gb300.plan" or header.get("version") != FORMAT_VERSION:
        raise ValueError(f"{path}: not a version-{FORMAT_VERSION} plan file")
    if pattern is None and A is not None:
        pattern = pattern_key(A)
    if pattern is not None:
        key = header.get("pattern")
        if key is None or key != pattern:
            raise ValueError(f"{path}: plan was made for a different sparsity pattern")

    spaces = []
    for j, rec in enumerate(header["spaces"]):
        kw = {}
        for name, info in rec["arrays"].items():
            if "arange" in info:
                kw[name] = np.arange(info["arange"], dtype=info["dtype"])
            else:
                kw[name] = arrays[f"s{j}.{name}"].astype(info["dtype"], copy=False)
        op = OpSpace(op_id=rec["op_id"], template=rec["template"], i_perm=kw.pop("i_perm"),
                     k_perm=kw.pop("k_perm"), idx_reordered=tuple(rec["idx_reordered"]),
                     hyb_short_begin_row=rec["hyb_short_begin_row"], TC_k_notsorted=rec["TC_k_notsorted"], **kw)
        if rec["kvals"]:
            kv = StoredKvals()
            blocks = arrays[f"s{j}.kv_block"]
            ptr = arrays[f"s{j}.kv_ptr"]
            pos, val, blen = arrays[f"s{j}.kv_pos"], arrays[f"s{j}.kv_val"], arrays[f"s{j}.kv_blen"]
            for n, b in enumerate(blocks):
                s, e = int(ptr[n]), int(ptr[n + 1])
                kv[int(b)] = StoredBlockOrder(pos[s:e], val[s:e], blen[n])
            op.blk_k_vals = kv
        m = rec["nnz_id_matrix"]
        if m is not None:
            mat = sp.csr_matrix((arrays[f"s{j}.nzm_data"].astype(m["dtype"], copy=False),
                                 arrays[f"s{j}.nzm_indices"], arrays[f"s{j}.nzm_indptr"]), shape=tuple(m["shape"]))
            mat.has_sorted_indices = m["sorted"]
            op.nnz_id_matrix = mat
        spaces.append(op)

    descs = [[_dec(x) for x in json.loads(d)] for d in header["descriptors"]]
    n = header["n_tiles"]
    g = {k[2:]: v for k, v in arrays.items() if k.startswith("t.")}
    ivs = _split(g["iv"], g["iv_len"])
    kvs = _split(g["kv"], g["kv_len"])
    kind = g["cov_kind"]
    row_lens = np.where(kind == 1, g["cov_row_len"], -1)
    nnz_lens = np.where(kind == 1, g["cov_nnz_len"], -1)
    indptrs = _split(g["cov_indptr"], row_lens)
    indices = _split(g["cov_indices"], nnz_lens)
    data = (None if header["cov_data_ones"] else _split(g["cov_data"], nnz_lens))
    vecs = _split(g["cov_vec"], np.where(kind == 2, g["cov_vec_len"], -1))
    ids = _split(g["ids"], np.where(g["has_ids"] == 1, g["ids_len"], -1))
    tiles = []
    for i in range(n):
        ts, params, bts, bparams = descs[int(g["desc"][i])]
        pos = tuple(Fraction(int(g["pos_num"][i, c]), int(g["pos_den"][i, c])) if g["pos_den"][i, c]
                    else int(g["pos_num"][i, c]) for c in range(int(g["pos_len"][i])))
        space, atomic, j_num, nnz = (int(x) for x in g["flags"][i])
        if kind[i] == 1:
            d = np.ones(len(indices[i])) if data is None else data[i]
            cov = sp.csr_matrix((d, indices[i], indptrs[i]), shape=tuple(int(x) for x in g["cov_shape"][i]))
        elif kind[i] == 2:
            cov = vecs[i]
        else:
            cov = None
        t = Tile(op=spaces[space], tile_sizes=ts, tile_pos=pos, params=params, best_tile_sizes=bts,
                 best_params=bparams, is_atomic=bool(atomic),
                 tile_i_rng=tuple(int(x) for x in g["i_rng"][i]) if g["rng_set"][i, 0] else None,
                 tile_k_rng=tuple(int(x) for x in g["k_rng"][i]) if g["rng_set"][i, 1] else None,
                 i_vals=ivs[i], k_vals=kvs[i], covered=cov,
                 pred_cost=None if np.isnan(g["pred"][i]) else float(g["pred"][i]),
                 nnz_when_selected=None if g["nnz_sel"][i] < 0 else int(g["nnz_sel"][i]), j_num=j_num, nnz=nnz)
        if ids[i] is not None:
            t.cov_ids = ids[i]
        tiles.append(t)
    return Plan(op_type=header["op_type"], shape=tuple(header["shape"]), tiles=tiles,
                max_bucket_size=header["max_bucket_size"], level_num=header["level_num"], meta=header["meta"])


# ---------------------------------------------------------------------------
# cache
# ---------------------------------------------------------------------------
def _settings_key(search_kwargs):
    """Canonical text of the search settings, the cost model included by its
    full parameters (and the learned network's, when one is attached)."""
    kw = dict(search_kwargs)
    cost = kw.pop("cost", None)
    parts = [json.dumps({k: repr(v) for k, v in sorted(kw.items())})]
    if cost is not None:
        parts.append(cost.to_json())
        mlp = getattr(cost, "mlp", None)
        if mlp is not None:
            parts.append(mlp.to_json())
    return "\n".join(parts)


class PlanCache:
    """Plans on disk under ``directory``, one file per (pattern, op type,
    dense width, search settings, format version)."""

    def __init__(self, directory: str):
        self.directory = str(directory)
        os.makedirs(self.directory, exist_ok=True)
        self.hits = 0
        self.misses = 0

    def path(self, op_type, A, width, search_kwargs, pattern=None):
        h = hashlib.sha1()
        for part in (f"v{FORMAT_VERSION}", op_type, str(int(width)), pattern or pattern_key(A),
                     _settings_key(search_kwargs)):
            h.update(part.encode("utf-8"))
            h.update(b"\0")
        return os.path.join(self.directory, f"{op_type}_{h.hexdigest()[:24]}.npz")

    def get_or_search(self, op_type, A, width, search_kwargs, search):
        """The cached plan for these inputs, else ``search()``'s plan, which
        is then stored.  A file that does not read back as a plan for this
        pattern is replaced."""
        key = pattern_key(A)
        path = self.path(op_type, A, width, search_kwargs, key)
        if os.path.exists(path):
            try:
                plan = load_plan(path, pattern=key)
                if plan.op_type == op_type and tuple(plan.shape) == tuple(A.shape):
                    self.hits += 1
                    return plan, "cache"
            except (ValueError, KeyError, OSError, EOFError, zipfile.BadZipFile):
                pass
        self.misses += 1
        plan = search()
        save_plan(plan, path, pattern=key)
        return plan, "search"
