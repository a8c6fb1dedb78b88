"""Seeded synthetic sparse matrices with the shapes, sizes and value
distributions of the five workloads this package is measured on.

The reference evaluates on public graph / pruned-weight datasets (OGB arxiv,
reddit, PruneBERT; technical_report.pdf p.8 Table 4) that are not available
offline; these generators stand in for them with the same sizes and
statistical structure.  Every generator is deterministic in ``seed``.

All generators return a ``scipy.sparse.csr_matrix`` with sorted, de-duplicated
column indices and float64 values.  Dense operands are created separately by
``dense_operand``.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp


def _discrete_power_law(rng, n, exponent, kmin, kmax):
    ks = np.arange(kmin, kmax + 1, dtype=np.float64)
    p = ks ** (-float(exponent))
    p /= p.sum()
    return rng.choice(np.arange(kmin, kmax + 1), size=n, p=p)


def _rows_without_replacement(rng, lens, ncols):
    """Column indices drawn uniformly without replacement for every row."""
    lens = np.minimum(np.asarray(lens, dtype=np.int64), ncols)
    indptr = np.zeros(len(lens) + 1, dtype=np.int64)
    np.cumsum(lens, out=indptr[1:])
    indices = np.empty(indptr[-1], dtype=np.int64)
    for r, n in enumerate(lens):
        if n == 0:
            continue
        if n * 4 < ncols:
            # rejection sampling is much faster than a full permutation
            cols = np.unique(rng.integers(0, ncols, size=int(n * 1.3) + 8))
            while len(cols) < n:
                cols = np.unique(np.concatenate([cols, rng.integers(0, ncols, size=n)]))
            cols = rng.permutation(cols)[:n]
        else:
            cols = rng.choice(ncols, size=n, replace=False)
        indices[indptr[r]:indptr[r + 1]] = np.sort(cols)
    return indptr, indices


def power_law_rows(m, k, exponent=2.1, min_len=1, max_len=1024, seed=0,
                   values="uniform"):
    """Rows whose lengths follow p(len) ~ len^-exponent on [min_len, max_len].

    ``values``: "uniform" -> U(-1, 1); "ones" -> 1.0.
    """
    rng = np.random.default_rng(seed)
    lens = _discrete_power_law(rng, m, exponent, min_len, min(max_len, k))
    indptr, indices = _rows_without_replacement(rng, lens, k)
    if values == "ones":
        data = np.ones(len(indices))
    else:
        data = rng.uniform(-1.0, 1.0, size=len(indices))
    A = sp.csr_matrix((data, indices, indptr), shape=(m, k))
    A.sort_indices()
    return A


def _chung_lu_edges(rng, n, exponent, avg_deg, max_deg):
    """Undirected edges with a power-law expected degree sequence."""
    dmin = 1
    w = _discrete_power_law(rng, n, exponent, dmin, max_deg).astype(np.float64)
    w *= avg_deg / w.mean()
    n_edges = int(round(w.sum() / 2))
    p = w / w.sum()
    u = rng.choice(n, size=n_edges, p=p)
    v = rng.choice(n, size=n_edges, p=p)
    keep = u != v
    return u[keep], v[keep]


def _planted_blocks(rng, n, n_blocks, bs_rows=16, bs_cols=16, density=(0.5, 0.9),
                    symmetric=True, offdiag_frac=0.5):
    """Dense-ish blocks aligned to bs_rows-row windows; columns aligned to bs_cols."""
    n_rwin = n // bs_rows
    n_cwin = n // bs_cols
    rows_out, cols_out = [], []
    for _ in range(n_blocks):
        rw = int(rng.integers(0, n_rwin))
        if rng.random() < offdiag_frac:
            cw = int(rng.integers(0, n_cwin))
        else:
            cw = min((rw * bs_rows) // bs_cols, n_cwin - 1)
        dens = rng.uniform(*density)
        mask = rng.random((bs_rows, bs_cols)) < dens
        r, c = np.nonzero(mask)
        rows_out.append(r + rw * bs_rows)
        cols_out.append(c + cw * bs_cols)
    r = np.concatenate(rows_out) if rows_out else np.zeros(0, np.int64)
    c = np.concatenate(cols_out) if cols_out else np.zeros(0, np.int64)
    if symmetric:
        r, c = np.concatenate([r, c]), np.concatenate([c, r])
    return r, c


def _to_pattern(n_rows, n_cols, r, c):
    A = sp.csr_matrix((np.ones(len(r)), (r, c)), shape=(n_rows, n_cols))
    A.sum_duplicates()
    A.data[:] = 1.0
    A.sort_indices()
    return A


def community_graph(n=169_343, target_nnz=1_170_000, exponent=2.0,
                    block_frac=0.30, max_deg=4096, seed=0, values="inv_deg",
                    block_density=(0.5, 0.9)):
    """Symmetric power-law graph plus planted 16x16 communities.

    About ``block_frac`` of the nonzeros fall in 16x16 blocks of density
    >= 0.5 aligned to 16-row windows; the rest is a Chung-Lu power-law graph
    with degree exponent ``exponent``.  Values are 1/deg(row) ("inv_deg") or 1.
    """
    rng = np.random.default_rng(seed)
    mean_dens = sum(block_density) / 2
    per_block = 2 * 256 * mean_dens  # symmetric -> two copies
    n_blocks = max(1, int(round(block_frac * target_nnz / per_block)))
    br, bc = _planted_blocks(rng, n, n_blocks, density=block_density)
    n_block_nnz = _to_pattern(n, n, br, bc).nnz
    remaining = max(0, target_nnz - n_block_nnz)
    # duplicates and self loops are dropped, so calibrate the edge budget once
    state = rng.bit_generator.state
    avg_deg = remaining / n
    for _ in range(2):
        rng.bit_generator.state = state
        u, v = _chung_lu_edges(rng, n, exponent, max(avg_deg, 1e-3), max_deg)
        r = np.concatenate([br, u, v])
        c = np.concatenate([bc, v, u])
        A = _to_pattern(n, n, r, c)
        if A.nnz == 0 or abs(A.nnz - target_nnz) < 0.01 * target_nnz:
            break
        avg_deg *= max(target_nnz - n_block_nnz, 1) / max(A.nnz - n_block_nnz, 1)
    if values == "inv_deg":
        deg = np.diff(A.indptr).astype(np.float64)
        A.data = np.repeat(1.0 / np.maximum(deg, 1.0), np.diff(A.indptr))
    return A


def pruned_weight(m=3072, k=768, sparsity=0.90, block_frac=0.5, std=0.02, seed=0):
    """Block-pruned + unstructured-pruned weight matrix.

    ``block_frac`` of the kept nonzeros are full 16x16 blocks on the 16x16
    grid; the rest are uniform random positions outside those blocks.
    Values N(0, std).
    """
    rng = np.random.default_rng(seed)
    keep = int(round(m * k * (1.0 - sparsity)))
    n_blk = int(round(keep * block_frac / 256))
    gm, gk = m // 16, k // 16
    blk_ids = rng.choice(gm * gk, size=n_blk, replace=False)
    dense = np.zeros((m, k), dtype=bool)
    for b in blk_ids:
        bi, bk = divmod(int(b), gk)
        dense[bi * 16:(bi + 1) * 16, bk * 16:(bk + 1) * 16] = True
    rest = keep - n_blk * 256
    free = np.flatnonzero(~dense.ravel())
    pick = rng.choice(free, size=rest, replace=False)
    dense.ravel()[pick] = True
    r, c = np.nonzero(dense)
    A = sp.csr_matrix((rng.normal(0.0, std, size=len(r)), (r, c)), shape=(m, k))
    A.sort_indices()
    return A


def sddmm_mask(n=100_000, target_nnz=2_000_000, exponent=2.1, block_frac=0.10,
               seed=0, max_len=4096):
    """Power-law rows plus ~``block_frac`` of nonzeros in dense 32x16 blocks."""
    rng = np.random.default_rng(seed)
    n_blocks = int(round(block_frac * target_nnz / 512))
    br, bc = _planted_blocks(rng, n, n_blocks, bs_rows=32, bs_cols=16,
                             density=(1.0, 1.0), symmetric=False, offdiag_frac=1.0)
    remaining = target_nnz - len(br)
    remaining *= 0.905  # power-law tail rows lose ~10% to duplicate columns
    # pick kmin so that the mean row length matches the remaining budget
    mean_target = remaining / n
    kmin = 1
    for cand in range(1, 64):
        ks = np.arange(cand, max_len + 1, dtype=np.float64)
        p = ks ** -exponent
        if (ks * p).sum() / p.sum() >= mean_target:
            kmin = cand
            break
    lens = _discrete_power_law(rng, n, exponent, kmin, max_len)
    lens = np.minimum(lens, n)
    rows = np.repeat(np.arange(n), lens)
    cols = rng.integers(0, n, size=len(rows))
    A = _to_pattern(n, n, np.concatenate([br, rows]), np.concatenate([bc, cols]))
    return A


def gcn_graph(n=232_965, target_nnz=11_600_000, exponent=1.9, block_frac=0.10,
              max_deg=8192, seed=0):
    """Symmetric power-law graph (degree exponent 1.9) with 16x16 communities,
    values normalised by 1/deg."""
    return community_graph(n=n, target_nnz=target_nnz, exponent=exponent,
                           block_frac=block_frac, max_deg=max_deg, seed=seed)


def dense_operand(rows, cols, seed=1, dist="normal", dtype=np.float32):
    rng = np.random.default_rng(seed)
    if dist == "normal":
        x = rng.standard_normal((rows, cols))
    else:
        x = rng.uniform(-1.0, 1.0, size=(rows, cols))
    return x.astype(dtype)


def logsparse_pattern(n):
    """LogSparse attention mask (Li et al., 2019), n x n: row i attends to
    itself, to i - 2^j for 2^j <= i and to i + 2^j for j <
    floor(log2(n - i - 1)) -- the definition of the reference's
    test_LogSparse (MY_sparse/gen_formats_v2.py:2926-2964).  Values 1."""
    rows, cols = [], []
    for i in range(n):
        back = [i - (1 << j) for j in range(int(math.log(i, 2)) + 1)] if i > 0 else []
        fwd = [i + (1 << j) for j in range(int(math.log(n - i - 1, 2)))] if i < n - 1 and n - i - 1 > 0 else []
        c = sorted(set(back + [i] + fwd))
        rows.extend([i] * len(c))
        cols.extend(c)
    return _to_pattern(n, n, np.asarray(rows), np.asarray(cols))


def strided_pattern(n):
    """Strided attention mask (Child et al., 2019), n x n with stride
    s = floor(sqrt(n)): row i attends to the window |i - j| < s and to
    i +- k s for 1 <= k < (n - 1 - i) / s (forward) and k < i / s (backward)
    -- the reference's test_Strided (MY_sparse/gen_formats_v2.py:2970-3003).
    Values 1."""
    s = int(n ** 0.5)
    rows, cols = [], []
    for i in range(n):
        c = set(range(max(i - s + 1, 0), min(i + s, n)))
        c.update(i + k * s for k in range(1, int((n - 1 - i) / s)))
        c.update(i - k * s for k in range(1, int(i / s)))
        c = sorted(c)
        rows.extend([i] * len(c))
        cols.extend(c)
    return _to_pattern(n, n, np.asarray(rows), np.asarray(cols))
