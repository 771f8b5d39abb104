"""Differentiable range-min over ragged rows.

Forward: the exact batched range-min (values and leftmost argmin) of the
queries of every row, one persistent launch of the batch engine; the
argmins are saved. Backward: grad_values[row_start + argmin[q]] +=
grad_out[q], a hand-written fp32-atomic scatter kernel of librmq.so
(rmq_batch_scatter_grad); argmins come from the forward, never recomputed.
The subgradient convention is the one of min(): the whole gradient of a
query goes to its leftmost minimum.

Neither direction allocates outside torch's allocator, so a full
forward + backward step can be captured in a CUDA graph once the plan
exists.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np
import torch

from .batch import RMQBatch

__all__ = ["RangeMinFunction", "RaggedRangeMin", "range_min"]


class RangeMinFunction(torch.autograd.Function):
    """values (flat float32 CUDA tensor of all rows), queries (int32 [q, 2],
    row-local, grouped by row as the plan says) -> (min values, argmin)."""

    @staticmethod
    def forward(ctx, values: torch.Tensor, queries: torch.Tensor, plan: RMQBatch):
        val, idx = plan.run(values.detach(), queries)
        ctx.save_for_backward(idx)
        ctx.plan = plan
        ctx.n = values.numel()
        ctx.mark_non_differentiable(idx)
        return val, idx

    @staticmethod
    def backward(ctx, grad_val: torch.Tensor, grad_idx: Optional[torch.Tensor]):
        (idx,) = ctx.saved_tensors
        grad_values = None
        if ctx.needs_input_grad[0]:
            grad_values = torch.zeros(ctx.n, dtype=torch.float32, device=idx.device)
            ctx.plan.scatter_grad(idx, grad_val.contiguous(), grad_values, accumulate=True)
        return grad_values, None, None


def range_min(values: torch.Tensor, queries: torch.Tensor, plan: RMQBatch):
    """Functional form: (min values, argmin) with gradients to ``values``."""
    return RangeMinFunction.apply(values, queries, plan)


class RaggedRangeMin(torch.nn.Module):
    """Range-min over rows of uneven length stored back to back in one flat
    tensor. ``row_lengths[i]`` elements form row i; ``queries_per_row[i]``
    consecutive queries of the query tensor belong to row i."""

    def __init__(self, row_lengths: Sequence[int], queries_per_row: Sequence[int],
                 bucket_bs: Optional[Sequence[int]] = None):
        super().__init__()
        lens = np.asarray(row_lengths, dtype=np.int64)
        qc = np.asarray(queries_per_row, dtype=np.int64)
        starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
        qstarts = np.concatenate([[0], np.cumsum(qc)[:-1]])
        self.n = int(lens.sum())
        self.q = int(qc.sum())
        self.plan = RMQBatch(starts, lens, qstarts, qc, bucket_bs)

    def forward(self, values: torch.Tensor, queries: torch.Tensor):
        if values.numel() != self.n or queries.shape[0] != self.q:
            raise ValueError("values / queries do not match the planned rows")
        return RangeMinFunction.apply(values, queries, self.plan)
