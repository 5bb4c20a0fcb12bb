"""Data parallelism over processes, one GPU each: the reference's ``pmap`` training step with
``psum`` of the gradient and the loss (solvers/poisson/trainer.py:716-834), and the per-device
batch layout of ``DatasetDict(x, batch_size, num_gpus)`` (data/data_management.py:79-159).

Residual points are independent, so the only exchange is one sum of the parameter gradient
(and of the loss) per step.  The sum runs through ``torch.distributed`` (NCCL between GPUs,
gloo between CPU processes).
"""

from __future__ import annotations

import math

import numpy as np
import torch


def device_batches(n_points: int, batch_size: int, num_gpus: int):
    """Slot layout of ``DatasetDict(x, batch_size, num_gpus)``.

    Each device owns a contiguous run of ceil(n/num_gpus) points cut into batches of
    ``bs = min(batch_size, ceil(n/num_gpus))`` points; a device whose run does not fold
    exactly gets one extra, padded batch (data_management.py:104-159).

    Returns (bs, layout) with layout[g][b] = (begin, end, n_pad): batch b of device g is
    points [begin, end) of the point array followed by n_pad padding points.
    """
    if n_points <= 0 or batch_size <= 0 or num_gpus <= 0:
        raise ValueError("device_batches: sizes must be positive")
    per_gpu = int(math.ceil(n_points / num_gpus))
    bs = min(batch_size, per_gpu)
    extra = 1 if per_gpu % bs else 0
    nb = per_gpu // bs
    last = per_gpu % bs
    layout = []
    for g in range(num_gpus):
        rows = []
        end = 0
        for b in range(nb):
            begin = g * (nb * bs + extra * last) + b * bs
            end = min(begin + bs, n_points)
            begin = min(begin, n_points)
            rows.append((begin, end, bs - (end - begin)))
        if extra:
            begin = end
            end = n_points if g == num_gpus - 1 else begin + last
            if end - begin > bs:
                raise ValueError("device_batches: the last device's extra batch overflows its batch size")
            rows.append((begin, end, bs - (end - begin)))
        layout.append(rows)
    return bs, layout


def device_points(points: np.ndarray, batch_size: int, rank: int, world: int, pad_fn):
    """The points of device ``rank`` in batch order (each batch ``bs`` points, padding from
    ``pad_fn(count)`` appended to short batches): an array of shape [n_batches * bs, 3]."""
    bs, layout = device_batches(points.shape[0], batch_size, world)
    parts = []
    for begin, end, n_pad in layout[rank]:
        parts.append(points[begin:end])
        if n_pad:
            parts.append(np.asarray(pad_fn(n_pad), points.dtype))
    return np.concatenate(parts).astype(points.dtype), bs, len(layout[rank])


def allreduce_sum_(grad: torch.Tensor, loss: torch.Tensor | None = None, group=None):
    """psum of the per-device gradient and loss (trainer.py:829-830), in place."""
    torch.distributed.all_reduce(grad, op=torch.distributed.ReduceOp.SUM, group=group)
    if loss is not None:
        torch.distributed.all_reduce(loss, op=torch.distributed.ReduceOp.SUM, group=group)
    return grad, loss
