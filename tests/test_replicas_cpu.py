"""Multi-rank host logic on CPU: member ranges per rank and the whole-job
throughput of replicas (sum of the ranks' units over the slowest rank's time),
over world_size-2 gloo process groups."""
import os
import socket

import pytest

from gpuocean_gb300.utils.replicas import ReplicaGroup, member_range


def test_member_ranges_cover_every_member_once():
    for n in (0, 1, 7, 256, 672):
        for world in (1, 2, 3, 8):
            covered = []
            for r in range(world):
                first, count = member_range(n, r, world)
                covered += list(range(first, first + count))
            assert covered == list(range(n))
            counts = [member_range(n, r, world)[1] for r in range(world)]
            assert max(counts) - min(counts) <= 1
    with pytest.raises(ValueError):
        member_range(4, 2, 2)


def test_single_rank_is_local():
    g = ReplicaGroup(world=1, rank=0)
    g.barrier()
    assert g.max(3.0) == 3.0 and g.sum(2.0) == 2.0
    assert g.throughput(10.0, 2.0) == 5.0
    g.close()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    g = ReplicaGroup(backend="gloo")
    g.barrier()
    first, count = member_range(256, g.rank, g.world)
    units = count * 153600.0                  # member-cells stepped by this rank
    seconds = 1.0 + rank                      # rank 1 is the slower one
    out[rank] = (g.max(seconds), g.sum(units), g.throughput(units, seconds), first, count)
    g.close()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as manager:
        out = manager.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for r in (0, 1):
        mx, total, rate, first, count = res[r]
        assert mx == 2.0
        assert total == 256 * 153600.0
        assert rate == pytest.approx(256 * 153600.0 / 2.0)
    assert (res[0][3], res[0][4], res[1][3], res[1][4]) == (0, 128, 128, 128)
