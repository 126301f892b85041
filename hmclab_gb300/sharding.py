"""Chains sharded over GPUs: one process per GPU, each running its own chains
(weak scaling, no collective in the sampling loop); only summaries cross
ranks, over whatever torch.distributed process group the caller set up.

The reference runs independent chains as forked processes
(`ParallelSampleSMP`, hmclab/Samplers.py:1807-1977) and never communicates
between them during sampling; here the unit of parallelism is a rank with a
batch of chains, and the per-rank results are combined at the end:

  rank_environment()       RANK / WORLD_SIZE / LOCAL_RANK from the launcher
  rank_seed(seed, rank)    a distinct Philox key per rank
  combine_ess(ess, sec)    sum of the per-rank multi-chain ESS and the
                           slowest rank's time (independent, stationary ranks)
  combine_moments(...)     pooled mean and standard deviation of all samples
"""
import os

import numpy as _np


def rank_environment():
    """(rank, world_size, local_rank) from the launcher's environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def rank_seed(seed, rank):
    """Philox key of a rank: ranks never share a counter stream."""
    return (int(seed) + 0x9E3779B97F4A7C15 * int(rank)) & 0xFFFFFFFFFFFFFFFF


def _gather(vec):
    import torch
    import torch.distributed as dist

    t = torch.as_tensor(_np.ascontiguousarray(vec, dtype=_np.float64))
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [t.numpy()]
    parts = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, t)
    return [p.numpy() for p in parts]


def combine_ess(ess, seconds):
    """ESS per parameter over all ranks and the time of the slowest rank.

    The per-rank multi-chain ESS values are added.  That equals the ESS of
    the pooled chains only when every rank's chains are independent and
    already stationary on the same target: the sum never sees the variance
    between ranks, so ranks that have not mixed (different modes, unfinished
    burn-in) make it overstate the pooled ESS, which a split-R-hat over the
    pooled chains would expose.  The sampler's ranks start from burned-in
    states with disjoint Philox keys, which is the case this estimate is for."""
    parts = _gather(_np.concatenate([_np.asarray(ess, _np.float64).reshape(-1), [float(seconds)]]))
    total = sum(p[:-1] for p in parts)
    return total, max(float(p[-1]) for p in parts)


def combine_moments(mean, std, count):
    """Pooled mean and standard deviation over ranks, each rank contributing
    `count` samples with per-parameter `mean` and (population) `std`."""
    d = _np.asarray(mean).size
    vec = _np.concatenate([[float(count)], _np.asarray(mean, _np.float64).reshape(-1),
                           _np.asarray(std, _np.float64).reshape(-1)])
    parts = _gather(vec)
    n = _np.array([p[0] for p in parts])
    means = _np.stack([p[1:1 + d] for p in parts])
    stds = _np.stack([p[1 + d:] for p in parts])
    N = n.sum()
    m = (n[:, None] * means).sum(axis=0) / N
    second = (n[:, None] * (stds**2 + means**2)).sum(axis=0) / N
    return m, _np.sqrt(_np.maximum(second - m * m, 0.0))
