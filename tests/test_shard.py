"""The N>1 path on the CPU: two gloo ranks each build the candidate pairs of
their strips; together the strips partition the job's MBR join, and the
job-level reduction takes the slowest rank's times and the sum of the pairs.
Strip membership of targets is exact: a target whose only far vertex crosses
a strip boundary still lands in the strip it reaches."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from farm_gb300 import polygons as P
from farm_gb300 import shard

SIDE = 40.0
N_SRC, N_TGT = 300, 900


def _params():
    return P.StarParams(dom_lo=0.0, dom_hi=SIDE, r_lo=0.05, r_hi=2.0, n_lo=16, n_hi=200, sigma=0.3)


def strip_pairs(seed, strip, n_strips):
    """Global (source, target) ids of one strip's candidate pairs."""
    prm = _params()
    s_idx = shard.strip_sources(P.centres(prm, seed, N_SRC), strip, n_strips, SIDE)
    S = P.generate_indices(prm, seed, s_idx)
    xext = shard.target_extents(P.centres(prm, seed + 1, N_TGT), P.radii(prm, seed + 1, N_TGT))
    t_idx = shard.strip_targets(S.mbrs(), xext)
    T = P.generate_indices(prm, seed + 1, t_idx)
    loc = P.mbr_join(S.mbrs(), T.mbrs())
    return np.stack([s_idx[loc[:, 0]], t_idx[loc[:, 1]]], axis=1).astype(np.int64)


def spike_strip_pairs(strip, n_strips):
    """One strip of the spike job (_spike_job), its targets chosen by their MBRs."""
    S, T = _spike_job()
    s_cent = np.array([[3.0, 10.0, 0.5], [15.0, 10.0, 1.0]])
    s_idx = shard.strip_sources(s_cent, strip, n_strips, 20.0).astype(np.int64)
    if len(s_idx) == 0:
        return np.zeros((0, 2), np.int64)
    ms, mt = S.mbrs()[s_idx], T.mbrs()
    t_idx = shard.strip_targets(ms, mt[:, [0, 2]]).astype(np.int64)
    loc = P.mbr_join(ms, mt[t_idx])
    return np.stack([s_idx[loc[:, 0]], t_idx[loc[:, 1]]], axis=1).astype(np.int64)


def _rank_main(rank, world, port, n_strips, seed, outdir, job="generator"):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard.strips_of_rank(rank, world, n_strips)
        per_strip = (lambda b: strip_pairs(seed, b, n_strips)) if job == "generator" else \
            (lambda b: spike_strip_pairs(b, n_strips))
        pairs = np.concatenate([per_strip(b) for b in mine])
        # a rank's times differ; the job takes the slowest
        t_dev, t_e2e = 1.0 + rank, 10.0 - rank
        out = shard.reduce_job(t_dev, t_e2e, len(pairs))
        np.save(os.path.join(outdir, f"pairs{rank}.npy"), pairs)
        np.save(os.path.join(outdir, f"job{rank}.npy"), np.array(out))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_strips_of_rank_round_robin():
    assert shard.strips_of_rank(0, 2, 5) == [0, 2, 4]
    assert shard.strips_of_rank(1, 2, 5) == [1, 3]
    assert shard.strips_of_rank(3, 4, 3) == []
    with pytest.raises(ValueError):
        shard.strips_of_rank(2, 2, 4)
    cover = sorted(b for r in range(3) for b in shard.strips_of_rank(r, 3, 10))
    assert cover == list(range(10))


def test_strip_sources_partition():
    c = np.random.default_rng(5).uniform(0, SIDE, (1000, 3))
    parts = [shard.strip_sources(c, b, 7, SIDE) for b in range(7)]
    allp = np.sort(np.concatenate(parts))
    assert np.array_equal(allp, np.arange(1000, dtype=np.uint64))
    with pytest.raises(ValueError):
        shard.strip_sources(c, 7, 7, SIDE)


def test_reduce_job_without_group():
    assert shard.reduce_job(2.0, 3.0, 17) == (2.0, 3.0, 17.0)


@pytest.mark.parametrize("n_strips", [2, 5])
def test_two_gloo_ranks_partition_the_join(host_built, tmp_path, n_strips):
    seed, world = 23, 2
    mp.start_processes(_rank_main, args=(world, _free_port(), n_strips, seed, str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    per = [np.load(tmp_path / f"pairs{r}.npy") for r in range(world)]
    jobs = [np.load(tmp_path / f"job{r}.npy") for r in range(world)]
    # every rank sees the same job figures: max times, summed pairs
    for j in jobs:
        assert j[0] == 2.0 and j[1] == 10.0 and j[2] == sum(len(p) for p in per)
    # the ranks' pairs are disjoint and their union is the whole job's join
    prm = _params()
    S, T = P.generate(prm, seed, N_SRC), P.generate(prm, seed + 1, N_TGT)
    full = P.mbr_join(S.mbrs(), T.mbrs()).astype(np.int64)
    key = lambda a: a[:, 0] * N_TGT + a[:, 1]
    got = np.concatenate([key(p) for p in per])
    assert len(np.unique(got)) == len(got)
    assert np.array_equal(np.sort(got), np.sort(key(full)))
    assert all(len(p) > 0 for p in per)


def test_generator_radii_bound_every_vertex(host_built):
    """target_extents() holds every stored vertex of every generated polygon."""
    prm = P.StarParams(dom_lo=0.0, dom_hi=419.0, r_lo=0.05, r_hi=2.0, n_lo=16, n_hi=3000, sigma=0.3)
    c, r = P.centres(prm, 77, 2000), P.radii(prm, 77, 2000)
    ext = shard.target_extents(c, r)
    m = P.generate(prm, 77, 2000).mbrs()
    assert (m[:, 0] >= ext[:, 0]).all() and (m[:, 2] <= ext[:, 1]).all()
    # and it is tight: the farthest vertex reaches within 1e-3 of the bound on some polygon
    far = np.maximum(c[:, 0] - m[:, 0], m[:, 2] - c[:, 0]) / r
    assert far.max() > 0.9


def _spike_job():
    """Two sources, one per strip of [0, 20) (boundary x = 10), and a target
    centred in strip 0 whose single far vertex crosses into strip 1 and
    overlaps source 1's MBR there; its other vertices stay near its centre."""
    sq = lambda cx, cy, h: np.array([[cx - h, cy - h], [cx + h, cy - h], [cx + h, cy + h], [cx - h, cy + h],
                                     [cx - h, cy - h]], np.float32)
    spike = np.array([[4.0, 9.0], [5.0, 9.0], [14.5, 10.0], [5.0, 11.0], [4.0, 11.0], [4.0, 9.0]], np.float32)
    mk = lambda rs: P.PolygonSet(np.concatenate([[0], np.cumsum([len(r) for r in rs])]).astype(np.uint64),
                                 np.ascontiguousarray(np.concatenate(rs), dtype=np.float32))
    S = mk([sq(3.0, 10.0, 0.5), sq(15.0, 10.0, 1.0)])
    T = mk([spike, sq(16.0, 13.0, 0.5)])
    return S, T


def test_far_vertex_crossing_a_strip_boundary(host_built):
    S, T = _spike_job()
    s_cent = np.array([[3.0, 10.0, 0.5], [15.0, 10.0, 1.0]])
    full = {tuple(p) for p in P.mbr_join(S.mbrs(), T.mbrs()).tolist()}
    assert (1, 0) in full  # the spike's far vertex reaches source 1
    mt = T.mbrs()
    got = set()
    for b in range(2):
        s_idx = shard.strip_sources(s_cent, b, 2, 20.0)
        t_idx = shard.strip_targets(S.mbrs()[s_idx.astype(np.int64)], mt[:, [0, 2]])
        loc = P.mbr_join(S.mbrs()[s_idx.astype(np.int64)], mt[t_idx.astype(np.int64)])
        got |= {(int(s_idx[a]), int(t_idx[c])) for a, c in loc.tolist()}
    assert got == full
    # a bound from the target's centre and a typical radius would have missed it
    centre_only = shard.strip_targets(S.mbrs()[[1]], np.array([[4.0, 6.0], [15.5, 16.5]]))
    assert 0 not in centre_only.tolist()


def test_two_gloo_ranks_spike_target(host_built, tmp_path):
    """Two gloo ranks, one strip each: the target whose far vertex crosses the
    strip boundary gives rank 1 its pair with source 1."""
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), 2, 0, str(tmp_path), "spike"), nprocs=world,
                       join=True, start_method="spawn")
    per = [np.load(tmp_path / f"pairs{r}.npy") for r in range(world)]
    S, T = _spike_job()
    full = {tuple(p) for p in P.mbr_join(S.mbrs(), T.mbrs()).tolist()}
    got = [{tuple(p) for p in a.tolist()} for a in per]
    assert not (got[0] & got[1])
    assert got[0] | got[1] == full
    assert (1, 0) in got[1]
