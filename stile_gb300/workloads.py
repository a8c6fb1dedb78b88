"""Seeded synthetic stand-ins for the five benchmark configurations.

The reference measures on OGB arxiv / reddit, PruneBERT weights and
sparse-attention masks, none of which is available offline.  Each function
here builds a matrix with the configuration's shape, nonzero count, degree
distribution, block structure and value distribution from
``stile_gb300.synthetic``, plus dense operands drawn N(0, 1):

  plain      config 1: 4096 x 4096 power-law rows (exponent 2.1, lengths
             1..1024; ``min_len=10`` gives the ~156k-nonzero variant),
             values U(-1, 1), B 4096 x 64, fp32 path
  graph      config 2: 169,343^2 symmetric graph, ~1.17M nonzeros, ~30% in
             16x16 blocks of density >= 0.5, values 1/deg, B 169,343 x 128
  pruned     config 3: W 3072 x 768 (``transposed``: 768 x 3072) at 90%
             sparsity, half of the kept nonzeros in 16x16 blocks, values
             N(0, 0.02); activations K x 4096 rounded to bf16
  sddmm      config 4: 100,000^2 mask, ~2M nonzeros, power-law rows plus
             10% in dense 32x16 blocks; X, Y 100,000 x 64
  gcn        config 5: 232,965^2 symmetric graph (exponent 1.9, ~11.4M
             nonzeros, 16x16 communities), values 1/deg, hidden width 128
             (``width=41`` for the second layer)
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import synthetic as syn


@dataclass
class Workload:
    name: str
    kind: str                 # "spmm" (forward + backward) or "sddmm"
    A: object                 # scipy CSR (the sparse matrix or the mask)
    width: int                # N (SpMM) or F (SDDMM)
    dense: dict = field(default_factory=dict)
    fp32: bool = False        # the fp32 path: split-bf16 tensor tiles
    note: str = ""


def _bf16_round(x):
    """float32 values rounded to the nearest bf16 (ties to even), kept as
    float32."""
    from .device import _bf16_bits_to_f32, _to_bf16_bits
    return _bf16_bits_to_f32(_to_bf16_bits(x)).reshape(np.shape(x))


def plain(min_len=1, seed=0):
    A = syn.power_law_rows(4096, 4096, exponent=2.1, min_len=min_len, max_len=1024, seed=seed)
    return Workload(f"plain_4096_min{min_len}", "spmm", A, 64,
                    {"B": syn.dense_operand(4096, 64, seed=1), "dC": syn.dense_operand(4096, 64, seed=2)},
                    fp32=True, note="config 1: plain SpMM, fp32 path")


def graph(seed=0):
    A = syn.community_graph(n=169_343, target_nnz=1_170_000, exponent=2.0, block_frac=0.30, seed=seed)
    return Workload("hybrid_graph_169343", "spmm", A, 128,
                    {"B": syn.dense_operand(A.shape[1], 128, seed=1),
                     "dC": syn.dense_operand(A.shape[0], 128, seed=2)},
                    note="config 2: hybrid graph, bf16 tensor tiles + fp32 row tiles")


def pruned(transposed=False, seed=0):
    m, k = (768, 3072) if transposed else (3072, 768)
    A = syn.pruned_weight(m, k, sparsity=0.90, block_frac=0.5, std=0.02, seed=seed)
    return Workload(f"pruned_{m}x{k}", "spmm", A, 4096,
                    {"B": _bf16_round(syn.dense_operand(k, 4096, seed=1)),
                     "dC": _bf16_round(syn.dense_operand(m, 4096, seed=2))},
                    note="config 3: pruned weight, bf16-valued activations")


def sddmm(seed=0):
    M = syn.sddmm_mask(n=100_000, target_nnz=2_000_000, exponent=2.1, block_frac=0.10, seed=seed)
    return Workload("sddmm_mask_100000", "sddmm", M, 64,
                    {"X": syn.dense_operand(100_000, 64, seed=1), "Y": syn.dense_operand(100_000, 64, seed=2)},
                    note="config 4: SDDMM on a sparse-attention-like mask, fp32")


def gcn(width=128, seed=0):
    A = syn.gcn_graph(n=232_965, target_nnz=11_600_000, exponent=1.9, block_frac=0.10, seed=seed)
    return Workload(f"gcn_232965_N{width}", "spmm", A, width,
                    {"B": syn.dense_operand(A.shape[1], width, seed=1),
                     "dC": syn.dense_operand(A.shape[0], width, seed=2)},
                    note="config 5: GCN layer on a reddit-sized graph, bf16 tensor tiles + fp32 row tiles")


BY_NAME = {
    "plain": lambda: plain(1),
    "plain_min10": lambda: plain(10),
    "graph": graph,
    "pruned": lambda: pruned(False),
    "pruned_t": lambda: pruned(True),
    "sddmm": sddmm,
    "gcn": lambda: gcn(128),
    "gcn_41": lambda: gcn(41),
}


def sddmm_fp64_sample(A, X, Y, n_sample=200_000, seed=0):
    """(entry ids, float64 <X[row], Y[col]>) for a seeded sample of A's
    stored entries in CSR order (the whole list when it is shorter)."""
    rng = np.random.default_rng(seed)
    nnz = A.nnz
    ids = np.arange(nnz) if nnz <= n_sample else np.sort(rng.choice(nnz, n_sample, replace=False))
    rows = np.searchsorted(A.indptr, ids, side="right") - 1
    cols = A.indices[ids]
    ref = np.einsum("ij,ij->i", np.asarray(X, np.float64)[rows], np.asarray(Y, np.float64)[cols])
    return ids, ref
