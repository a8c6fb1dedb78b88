"""CPU oracle: the arithmetic of the reference's fused SpMM / SDDMM kernels,
restated in numpy over the reference-layout device arrays.

TEST INFRASTRUCTURE ONLY.  Nothing in the ``stile_gb300`` package imports this
module; it is used by ``tests/``, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py`` as the checker, never as the computation.

The reference never ran these kernels on a CPU: they are TVMScript templates
compiled by SparseTIR.  The semantics below follow the template definitions
and the atomic rewrite of the generated CUDA:

* ELL tile    -- ``my_fuse_formats.py:1162-1291`` (definition),
                 ``nvcc.py:291-319, 402-423`` (atomicAdd for atomic tiles):
                 ``C[I_out[r], j] (+)= sum_k A[r, k] * B[K_out[r, k], j]``
* TC tile     -- ``my_fuse_formats.py:1444-1520``: per compressed row block
                 ``io``, ``C[rows(io), j] (+)= sum_{blk in indptr[io]..}
                 A[blk] @ B[indices[blk], j]`` where ``rows(io)`` is
                 ``i_indices[io, :]`` when rows are reordered or the format is
                 atomic, else ``i_indices[io]*16 + 0..15``.
* 1D SDDMM    -- ``my_fuse_formats.py:2263-2317``: ``c1d[t] =
                 <X[mid[t]], Y[jidx[t]]>``, scattered by ``remap``.
* TC SDDMM    -- ``my_fuse_formats.py:2324-2415``: ``Cblk = X[i_idx[b]] @
                 Y[j_idx[b]]^T`` sampled at ``indicesDense`` into output
                 positions ``indices``; host reorder ``order_output_BSDDMM``
                 (``my_fuse_formats.py:4247-4288``).

Non-atomic ("owned") rows are stored and atomic rows accumulated; the
reference guarantees that an owned row has exactly one writer
(``ComputeTile.check_atomic``, gen_formats_v2.py:2414-2431, and the withdraw
post-processing, my_branch_and_bound.py:1652-1702).  ``spmm_from_arrays``
applies the stores first and the atomic adds second and reports any owned row
written twice with different values.
"""
from __future__ import annotations

import json

import numpy as np
import scipy.sparse as sp


# ---------------------------------------------------------------------------
# plain FP64 references (scipy CSR times dense; masked dot products)
# ---------------------------------------------------------------------------
def spmm_fp64(A, B):
    """C = A @ B in float64 (the reference's accuracy check,
    my_fuse_formats.py:4197-4214, uses scipy's ``A.dot(B)``)."""
    A = sp.csr_matrix(A, dtype=np.float64)
    return np.asarray(A @ np.asarray(B, dtype=np.float64))


def sddmm_fp64(A, X, Y):
    """out[t] = <X[row(t)], Y[col(t)]> for every stored nonzero t of A in CSR
    order (DGL ``u_dot_v`` semantics used as the reference's golden,
    my_fuse_formats.py:4331-4341)."""
    A = sp.csr_matrix(A)
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    return np.einsum("ij,ij->i", X[rows], Y[A.indices])


def rel_fro(x, ref):
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (den if den > 0 else 1.0))


# ---------------------------------------------------------------------------
# reference-layout executors
# ---------------------------------------------------------------------------
def _params(fmt):
    p = fmt["params"]
    return json.loads(p) if isinstance(p, str) else p


def _tile_extent(ts):
    """prod(tile_sizes[d][1:]) as used throughout the reference."""
    out = 1
    for v in ts[1:]:
        out *= int(v)
    return out


def spmm_from_arrays(formats, fmt_args, B, out_shape, check_owned=True):
    """Execute a fused SpMM described by reference-layout arrays.

    formats  : list of dicts with keys ``template`` ("sparse_template_ell" or
               "TensorCore_template"), ``tile_sizes`` and ``params``.
    fmt_args : per format, the tuple of arrays ``prepare_inputs_BSPMM``
               emits (my_fuse_formats.py:3321-3537):
               ELL -> (a, indices_k, indices_reordered_i)
               TC  -> (a, i_indices, indptr, indices); ``indices`` is
                      [blocks, klen] columns, or, for TC_k_notsorted
                      tiles, one k-block position per block whose columns
                      are [p * klen, (p + 1) * klen) (:3501-3502)
    B        : dense [K, max_j] (zero-padded columns allowed).
    Returns C [out_shape] in float64 and the list of owned-row conflicts.
    """
    B = np.asarray(B, dtype=np.float64)
    max_i, max_j = out_shape
    if B.shape[1] < max_j:
        B = np.concatenate([B, np.zeros((B.shape[0], max_j - B.shape[1]))], axis=1)
    C = np.zeros((max_i, max_j))
    stores = []   # (rows, partial)
    adds = []
    for fmt, args in zip(formats, fmt_args):
        p = _params(fmt)
        atomic = bool(p.get("real_atomic", False))
        if fmt["template"] == "sparse_template_ell":
            a, k_out, i_out = (np.asarray(x) for x in args)
            ilen = _tile_extent(fmt["tile_sizes"][0])
            klen = _tile_extent(fmt["tile_sizes"][2])
            a = a.reshape(-1, klen).astype(np.float64)
            k_out = k_out.reshape(-1, klen)
            part = np.einsum("rk,rkj->rj", a, B[k_out])
            rows = i_out.reshape(-1)
            assert a.shape[0] == rows.shape[0] == (a.shape[0] // ilen) * ilen
            (adds if atomic else stores).append((rows, part, a))
        elif fmt["template"] == "TensorCore_template":
            a, i_idx, indptr, indices = (np.asarray(x) for x in args)
            a = a.astype(np.float64)
            tsz = int(fmt["tile_sizes"][0][1])
            mb = len(indptr) - 1
            if indices.ndim == 1:
                klen = a.shape[2]
                cols = indices[:, None] * klen + np.arange(klen)[None, :]
                if cols.size and cols.max() >= B.shape[0]:
                    B = np.concatenate([B, np.zeros((int(cols.max()) + 1 - B.shape[0], B.shape[1]))])
                indices = cols
            part = np.zeros((mb, tsz, max_j))
            for io in range(mb):
                for blk in range(indptr[io], indptr[io + 1]):
                    part[io] += a[blk] @ B[indices[blk]]
            if i_idx.ndim == 2:
                rows = i_idx.reshape(-1)
            else:
                rows = (i_idx[:, None] * tsz + np.arange(tsz)[None, :]).reshape(-1)
            part = part.reshape(-1, max_j)
            (adds if atomic else stores).append((rows, part, None))
        else:
            raise ValueError(fmt["template"])
    conflicts = []
    written = {}
    for rows, part, a in stores:
        for r in range(len(rows)):
            row = int(rows[r])
            # a padded ELL row (all-zero values) stores zeros; C is
            # zero-initialised, so it only matters if it hits an owned row
            if a is not None and not np.any(a[r]):
                if row in written and np.any(written[row]):
                    conflicts.append(row)
                continue
            if row in written and check_owned:
                conflicts.append(row)
            C[row] = part[r]
            written[row] = part[r]
    for rows, part, _ in adds:
        np.add.at(C, rows, part)
    return C, conflicts


def sddmm_from_arrays(formats, fmt_args, X, Y, nnz):
    """Execute a fused SDDMM described by reference-layout arrays with the
    host-side output reorder (REMAP=False path).

    1D  -> (mid_idx, j_idx, remap, c1d_placeholder)
    TC  -> (i_indices, j_indices, indptr, indicesDense, indices, cTC_placeholder)
    Returns out [nnz] in float64 (CSR nonzero order of the original mask).
    """
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    out = np.zeros(nnz)
    tc_parts = []
    one_d = []
    for fmt, args in zip(formats, fmt_args):
        if fmt["template"] == "1D_sddmm":
            mid, jidx, remap = (np.asarray(x) for x in args[:3])
            c1d = np.einsum("tf,tf->t", X[mid], Y[jidx])
            one_d.append((remap, c1d))
        elif fmt["template"] == "TC_sddmm":
            i_idx, j_idx, indptr, dense_pos, indices = (np.asarray(x) for x in args[:5])
            nb = int(fmt["tile_sizes"][2][1])
            blocks = np.einsum("bmf,bnf->bmn", X[i_idx], Y[j_idx])
            flat = blocks.reshape(len(blocks), -1)
            for b in range(len(blocks)):
                sl = slice(indptr[b], indptr[b + 1])
                dp = dense_pos[sl]
                vm, vn = dp // nb, dp % nb
                tc_parts.append((indices[sl], blocks[b][vm, vn]))
            del flat
        else:
            raise ValueError(fmt["template"])
    # order_output_BSDDMM: TC results first, then the 1D results overwrite
    for idx, vals in tc_parts:
        out[idx] = vals
    for remap, c1d in one_d:
        out[remap] = c1d
    return out


# ---------------------------------------------------------------------------
# golden fixture access
# ---------------------------------------------------------------------------
def load_fixture(path):
    z = np.load(path, allow_pickle=False)
    meta = json.loads(bytes(z["meta"]).decode())
    arrays = {k: z[k] for k in z.files if k != "meta"}
    return meta, arrays


def fixture_args(meta, arrays):
    """Group the emitted argument arrays of a fixture per format, restoring
    the all-zero output placeholders that were stored by shape only."""
    n_dense = len(meta["dense_arg_shapes"])
    zero = meta.get("zero_args", {})
    flat = []
    for n in range(n_dense, meta["n_args"]):
        if f"arg{n}" in arrays:
            flat.append(arrays[f"arg{n}"])
        else:
            flat.append(np.zeros(zero[str(n)], dtype=np.float32))
    per_fmt = []
    pos = 0
    for f in meta["formats"]:
        t = f["template"]
        n = {"sparse_template_ell": 3, "TensorCore_template": 4,
             "1D_sddmm": 4, "TC_sddmm": 6}[t]
        per_fmt.append(tuple(flat[pos:pos + n]))
        pos += n
    assert pos == len(flat)
    return per_fmt


def fixture_matrix(meta, arrays):
    M, _, K = meta["idx_lens"]
    indptr = arrays["A_indptr"]
    indices = arrays["A_indices"]
    return sp.csr_matrix((np.ones(len(indices)), indices, indptr), shape=(M, K))
