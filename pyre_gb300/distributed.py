"""Sample-range sharding of one frame across ranks (one process per GPU).

Every sample is seeded by pixel_seed(x, y, s) (crates/pyre/src/sampler.rs:41-49),
so rank r can render samples [base + r*k, base + (r+1)*k) of the same frame
independently; there is no exchange on the data path. The per-rank films
(means over k samples) combine into the frame's mean with one sum-reduction
after rendering, outside any timed region.
"""
from __future__ import annotations

import numpy as np


def sample_range(rank: int, spp_per_rank: int, spp_base: int = 0) -> tuple[int, int]:
    start = spp_base + rank * spp_per_rank
    return start, start + spp_per_rank


def reduce_film_means(channels: dict, count: int, group=None) -> dict:
    """Combines per-rank per-pixel means of `count` samples into global means.

    `channels` maps names to numpy arrays (or torch tensors); works with any
    torch.distributed backend (gloo on CPU, NCCL on GPU tensors).
    """
    import torch
    import torch.distributed as dist

    out = {}
    n = torch.tensor([float(count)], dtype=torch.float64)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    for name, arr in channels.items():
        t = torch.as_tensor(np.asarray(arr) if not isinstance(arr, torch.Tensor) else arr).to(torch.float64)
        t = t * float(count)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out[name] = (t / n.item()).to(torch.float32).numpy() if t.device.type == "cpu" else t / n.item()
    return out


def reduce_gradients(mat_grad, env_grad, count: int, group=None):
    """Combines per-rank adjoint gradients into the gradient of the whole frame.

    Rank r's backward pass differentiates the mean of its own `count` samples,
    and the frame is the count-weighted mean of the ranks' films, so the
    frame's gradient is sum_r count_r * g_r / sum_r count_r. This is one sum
    all-reduce per step over the material gradients (FP64, n_materials x 6)
    and the environment texel gradients (FP32, h x w x 3, or None).
    Returns (mat_grad, env_grad) in the dtypes given.
    """
    import torch
    import torch.distributed as dist

    n = torch.tensor([float(count)], dtype=torch.float64)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    out = []
    for g, dtype in ((mat_grad, torch.float64), (env_grad, torch.float32)):
        if g is None:
            out.append(None)
            continue
        t = torch.as_tensor(np.asarray(g) if not isinstance(g, torch.Tensor) else g).to(dtype) * float(count)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        t = t / n.item()
        out.append(t.numpy() if t.device.type == "cpu" else t)
    return out[0], out[1]
