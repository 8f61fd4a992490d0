"""Cross-rank bookkeeping of independent replicas (one process per GPU under torchrun):
the per-block gather of driver.py:262-296, done with torch.distributed collectives on
whichever backend the process group uses (NCCL on GPUs, gloo on CPU), and the max-over-ranks
timing of the benchmark. The walker propagation itself has no cross-rank step: each rank
runs its own walkers; there is no global SR across ranks."""

from __future__ import annotations

from typing import Tuple

import torch
import torch.distributed as dist


def _active() -> bool:
    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def _device() -> torch.device:
    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")


def max_over_ranks(x: float) -> float:
    """The largest x over the ranks (every rank gets it); x itself on one rank."""
    if not _active():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_block(block_weight: float, block_energy: float,
                 block_observable: float = 0.0) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor, float]:
    """Every rank's (block weight, block energy, block observable) in rank order, and the
    block energy of the whole population sum(w E) / sum(w) (driver.py:275-296 gathers to rank
    0 and broadcasts that energy; an all-gather gives every rank both). Float64 CPU tensors
    [world] and a float."""
    t = torch.tensor([float(block_weight), float(block_energy), float(block_observable)], dtype=torch.float64)
    if _active():
        t = t.to(_device())
        parts = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
        dist.all_gather(parts, t)
        g = torch.stack(parts).cpu()
    else:
        g = t.reshape(1, 3)
    w, e, o = g[:, 0], g[:, 1], g[:, 2]
    return w, e, o, float(torch.sum(w * e) / torch.sum(w))
