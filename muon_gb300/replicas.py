"""Replicas on several GPUs: the host logic of multi-GPU rendering.

Pixel samples are independent, so N GPUs render without exchanging anything
while they work: each rank renders its own range of the sample indices of
the same frame (the counter-based RNG is keyed by the sample index, so the
ranges together are exactly the samples one GPU would render), and the FP64
films merge by addition at the end. The reference renders on the host
threads of one machine (muon/renderer.cc:28-80, tiles per thread); this
module is the multi-GPU counterpart of that split.

Works with any torch.distributed backend: NCCL for device films, gloo for
host tensors (the CPU tests).
"""
from __future__ import annotations


def sample_range(rank: int, world: int, spp: int) -> tuple[int, int]:
    """(sample_offset, pixel_samples) of `rank`'s share of `spp` samples per
    pixel: contiguous ranges, the first spp % world ranks one sample longer."""
    if world < 1 or not 0 <= rank < world or spp < 0:
        raise ValueError("bad rank, world size or sample count")
    base, extra = divmod(spp, world)
    count = base + (1 if rank < extra else 0)
    offset = rank * base + min(rank, extra)
    return offset, count


def merge_films(sum_, sum_sq, count, group=None) -> None:
    """Adds the ranks' films in place (all-reduce SUM of the FP64 sums, sums of
    squares and the sample counts); every rank ends with the whole film."""
    import torch.distributed as dist

    for t in (sum_, sum_sq, count):
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)


def reduce_step(device_ms: float, counted: float, device=None, group=None) -> tuple[float, float]:
    """Whole-job timing of a step: the slowest rank's device time and the sum
    of the rays every rank counted."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([device_ms, float(counted)], dtype=torch.float64, device=device)
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(t[0]), float(t[1])
    tmax, tsum = t.clone(), t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM, group=group)
    return float(tmax[0]), float(tsum[1])
