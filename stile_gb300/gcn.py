"""Two-layer graph convolution over one sparse adjacency, the differentiable
sparse layer the GCN workload trains (a 232,965-node graph, features
602 -> 128 -> 41):

    H1 = A (X W1),  Z1 = relu(H1),  H2 = A (Z1 W2)

Both products with A run through ``HybridSpMMFunction``: the forward is the
hybrid-tile SpMM, the backward dvals = SDDMM(dH, XW) over the forward tiles
and d(XW) = A^T dH with the transposed plan.  A's values are one tensor
shared by the two layers (their value gradients add up), each layer has its
own plan (the plan depends on the dense width).  The dense products X W1
and Z1 W2 are ordinary torch GEMMs; widths that are not a multiple of 4 are
computed into a zero-padded weight so that the SpMM operand rows stay
16-byte aligned without a copy per call.
"""
from __future__ import annotations

import torch

from .api import HybridSpMMFunction, PlanConfig, SpmmOperator


def _pad4(n: int) -> int:
    return (n + 3) // 4 * 4


class AlignedLinear(torch.nn.Module):
    """x @ W for W [fin, fout], returned as a [rows, fout] view of a
    [rows, ceil4(fout)] product (the extra weight columns are zero and not
    trained), so that its row stride is a multiple of 4 elements."""

    def __init__(self, weight: torch.Tensor):
        super().__init__()
        self.fout = weight.shape[1]
        self.weight = torch.nn.Parameter(weight.detach().clone())

    def forward(self, x):
        pad = _pad4(self.fout) - self.fout
        w = torch.nn.functional.pad(self.weight, (0, pad)) if pad else self.weight
        return (x @ w)[:, : self.fout]


class TwoLayerGCN(torch.nn.Module):
    """The two-layer GCN step on the GPU.  ``A`` is the scipy CSR adjacency
    (its values are the initial edge weights), W1 [fin, hidden], W2
    [hidden, fout]; ``cfg`` the plan settings of both layers."""

    def __init__(self, A, W1: torch.Tensor, W2: torch.Tensor, cfg: PlanConfig | None = None,
                 ops: tuple[SpmmOperator, SpmmOperator] | None = None):
        super().__init__()
        hidden, fout = W1.shape[1], W2.shape[1]
        if ops is None:
            ops = (SpmmOperator(A, hidden, cfg), SpmmOperator(A, fout, cfg))
        self.op1, self.op2 = ops
        dev = W1.device
        self.vals = torch.nn.Parameter(torch.as_tensor(self.op1.A.data, dtype=torch.float32, device=dev))
        self.lin1 = AlignedLinear(W1)
        self.lin2 = AlignedLinear(W2)

    def forward(self, X):
        H1 = HybridSpMMFunction.apply(self.vals, self.lin1(X), self.op1)
        Z1 = torch.relu(H1)
        return HybridSpMMFunction.apply(self.vals, self.lin2(Z1), self.op2)
