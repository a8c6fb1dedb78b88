"""Float64 restatement of sparse attention for checking the GPU pipeline
(test infrastructure: only tests import it).

* Patterns: the reference's LogSparse and Strided masks, restated loop for
  loop from MY_sparse/gen_formats_v2.py:2926-2964 (test_LogSparse) and
  :2970-3003 (test_Strided): per row, a list of columns, made unique and
  sorted.
* Attention: per head, scores s_t = scale * <Q[row(t)], K[col(t)]> on the
  pattern, softmax over each row's entries (the entries outside the pattern
  count as -inf, as in the reference's softmax check,
  my_3rdparty/Magicube/Magicube1/end2end_eval/sparse_transformer_magicube/
  verify/bsoftmax.py), out = P @ V.
"""
import math

import numpy as np
import scipy.sparse as sp


def logsparse_rows(n):
    rows = []
    for i in range(n):
        if i == 0:
            tmp = [i] + [i + 2 ** j for j in range(int(math.log(n - i - 1, 2)))]
        elif i == n - 1:
            tmp = [i - 2 ** j for j in range(int(math.log(i, 2)), -1, -1)] + [i]
        else:
            tmp = ([i - 2 ** j for j in range(int(math.log(i, 2)), -1, -1)] + [i]
                   + [i + 2 ** j for j in range(int(math.log(n - i - 1, 2)))])
        rows.append(np.unique(tmp))
    return rows


def strided_rows(n):
    s = int(n ** 0.5)
    rows = []
    for i in range(n):
        tmp = (list(range(max(i - s + 1, 0), min(i + s, n))) + [i + j * s for j in range(1, int((n - 1 - i) / s))]
               + [i - j * s for j in range(1, int(i / s))])
        rows.append(np.unique(tmp))
    return rows


def rows_to_csr(rows, n):
    indptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])])
    indices = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    return sp.csr_matrix((np.ones(len(indices)), indices, indptr), shape=(n, n))


def attention_fp64(pattern, Q, K, V, scale):
    """[H, n, Fv] float64 sparse attention over the CSR pattern."""
    A = sp.csr_matrix(pattern)
    Q, K, V = (np.asarray(x, np.float64) for x in (Q, K, V))
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    out = np.zeros((Q.shape[0], A.shape[0], V.shape[2]))
    for h in range(Q.shape[0]):
        s = scale * np.einsum("ij,ij->i", Q[h][rows], K[h][A.indices])
        p = np.empty_like(s)
        for r in range(A.shape[0]):
            a, b = A.indptr[r], A.indptr[r + 1]
            if b > a:
                e = np.exp(s[a:b] - s[a:b].max())
                p[a:b] = e / e.sum()
        out[h] = sp.csr_matrix((p, A.indices, A.indptr), shape=A.shape) @ V[h]
    return out
