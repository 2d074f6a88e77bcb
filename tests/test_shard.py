"""The N>1 path on the CPU: two gloo ranks each build the candidate pairs of
their strips; together the strips partition the job's MBR join, and the
job-level reduction takes the slowest rank's times and the sum of the pairs."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from farm_gb300 import polygons as P
from farm_gb300 import shard

SIDE = 40.0
N_SRC, N_TGT = 300, 900
EXTENT_RADII = float(np.exp(0.3 * 6.5))


def _params():
    return P.StarParams(dom_lo=0.0, dom_hi=SIDE, r_lo=0.05, r_hi=2.0, n_lo=16, n_hi=200, sigma=0.3)


def strip_pairs(seed, strip, n_strips):
    """Global (source, target) ids of one strip's candidate pairs."""
    prm = _params()
    s_idx = shard.strip_sources(P.centres(prm, seed, N_SRC), strip, n_strips, SIDE)
    S = P.generate_indices(prm, seed, s_idx)
    t_idx = shard.strip_targets(S.mbrs(), P.centres(prm, seed + 1, N_TGT), EXTENT_RADII)
    T = P.generate_indices(prm, seed + 1, t_idx)
    loc = P.mbr_join(S.mbrs(), T.mbrs())
    return np.stack([s_idx[loc[:, 0]], t_idx[loc[:, 1]]], axis=1).astype(np.int64)


def _rank_main(rank, world, port, n_strips, seed, outdir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard.strips_of_rank(rank, world, n_strips)
        pairs = np.concatenate([strip_pairs(seed, b, n_strips) for b in mine])
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
