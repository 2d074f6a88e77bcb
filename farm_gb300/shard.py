"""Weak-scaling shards of the polygon join: strips of the domain across ranks.

Candidate pairs are independent units (the reference hands them to threads
one index range at a time, query_context.cpp:145-160, and to its GPU kernels
one thread per pair, query_intersect.cu), so a job over a source set S and a
target set T splits with no exchange on the data path:

* the domain is cut into vertical strips by source centre; strip b holds the
  sources whose centre x lies in [b w, (b + 1) w), w = L / n_strips;
* strip b takes every target whose x-extent (an interval that holds all its
  vertices: the generator's exact largest radius about the centre, or the
  MBR itself) reaches the x-range of the strip's source MBRs;
* the strip's candidates are the MBR-overlapping pairs of those two sets.

Each candidate pair (s, t) of the whole job falls in the strip of s, and t
is always in that strip's target set (its MBR lies inside its x-extent and
overlaps the MBR of s), so the strips' pair sets partition the job's. Rank r runs strips
r, r + N, r + 2N, ...; the only collective is the reduction of the ranks'
pair counts and times at the end of a run.
"""
from __future__ import annotations

import numpy as np


def strips_of_rank(rank: int, world: int, n_strips: int) -> list[int]:
    """Strips rank `rank` of `world` runs, round robin."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    return list(range(rank, n_strips, world))


def strip_sources(src_centres: np.ndarray, strip: int, n_strips: int, side: float) -> np.ndarray:
    """Indices (uint64) of the sources centred in strip `strip` of a domain [0, side)."""
    if not 0 <= strip < n_strips:
        raise ValueError(f"strip {strip} outside 0..{n_strips - 1}")
    w = side / n_strips
    x = src_centres[:, 0]
    hi = (x < (strip + 1) * w) if strip + 1 < n_strips else np.ones(len(x), bool)
    lo = (x >= strip * w) if strip > 0 else np.ones(len(x), bool)
    return np.nonzero(lo & hi)[0].astype(np.uint64)


def target_extents(tgt_centres: np.ndarray, tgt_rmax: np.ndarray) -> np.ndarray:
    """Closed x-intervals [lo, hi] (float64 [n, 2]) that contain every vertex
    of each target: centre x -+ its largest vertex distance from the centre,
    widened by the float32 rounding of the stored coordinates (a relative
    2^-24 of the coordinate, bounded here by 1e-6 of |x| + 1e-6)."""
    cx = tgt_centres[:, 0]
    r = np.asarray(tgt_rmax, dtype=np.float64) * (1.0 + 1e-6)
    pad = 1e-6 * (np.abs(cx) + r + 1.0)
    return np.stack([cx - r - pad, cx + r + pad], axis=1)


def strip_targets(src_mbrs: np.ndarray, tgt_xext: np.ndarray) -> np.ndarray:
    """Indices (uint64) of the targets whose x-extent (tgt_xext[k] = [lo, hi],
    an interval holding every vertex of target k, e.g. target_extents() or the
    exact MBRs) reaches the x-range of the strip's source MBRs. A target
    outside that range has an MBR disjoint from every source MBR of the
    strip, so no candidate pair of the strip is lost."""
    if len(src_mbrs) == 0:
        return np.zeros(0, np.uint64)
    xlo, xhi = src_mbrs[:, 0].min(), src_mbrs[:, 2].max()
    return np.nonzero((tgt_xext[:, 1] >= xlo) & (tgt_xext[:, 0] <= xhi))[0].astype(np.uint64)


def reduce_job(t_dev: float, t_e2e: float, n_pairs: int, device=None) -> tuple[float, float, float]:
    """Whole-job figures over the default process group: the slowest rank's
    device and end-to-end times, and the pairs all ranks processed. With one
    process (no group) the inputs come back unchanged. `device` is where the
    backend reduces (a CUDA device for NCCL, None for gloo on the CPU)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(t_dev), float(t_e2e), float(n_pairs)
    tt = torch.tensor([t_dev, t_e2e], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(n_pairs)], dtype=torch.float64, device=device)
    dist.all_reduce(n)
    a, b = tt.tolist()
    return a, b, float(n.item())
