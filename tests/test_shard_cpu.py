"""CPU checks of the sharding of independent bubbles across ranks: the
partition of the ensemble and of the serving stream, and the host-side
bookkeeping of a multi-rank run (barriers, units summed, the slowest rank's
time) as two gloo processes, world_size 2."""
import os
import socket
import time

import numpy as np
import pytest

from soapbubble_gb300 import serve, shard, synth


def _check_partition(weights, world):
    parts = shard.partition(weights, world)
    assert len(parts) == world
    flat = sorted(k for p in parts for k in p)
    assert flat == list(range(len(weights)))
    loads = [sum(weights[k] for k in p) for p in parts]
    avg = sum(weights) / world
    assert max(loads) <= avg + max(weights, default=0) + 1e-9
    assert parts == shard.partition(weights, world)  # deterministic
    return parts, loads


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_ensemble_partition_is_complete_and_balanced(world):
    members = synth.ensemble(0)
    parts, loads = _check_partition([shard.member_weight(m.nTheta) for m in members], world)
    shards = [shard.shard_members(members, world, r) for r in range(world)]
    assert sum(len(s) for s in shards) == len(members)
    # the ensemble's cells are dominated by its 512 x 1024 members: every rank
    # gets a share within one largest member of the average
    assert max(loads) - min(loads) <= shard.member_weight(512)


def test_partition_edge_cases():
    assert shard.partition([], 3) == [[], [], []]
    assert shard.partition([5.0], 3) == [[0], [], []]
    assert shard.partition([1.0, 1.0, 1.0, 1.0], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard.partition([1.0], 0)


def test_request_shards_keep_arrival_order():
    reqs = serve.make_requests(200, 20.0, seed=3)
    got = []
    for r in range(3):
        mine = shard.shard_requests(reqs, 3, r)
        assert [q.arrival for q in mine] == sorted(q.arrival for q in mine)
        got += [q.rid for q in mine]
    assert sorted(got) == list(range(200))
    _check_partition([shard.member_weight(q.nTheta, q.steps) for q in reqs], 3)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    ranks = shard.Ranks("gloo")
    members = synth.ensemble(0)
    mine = shard.shard_members(members, ranks.world, ranks.rank)
    units = float(sum(shard.member_weight(m.nTheta) for m in mine))

    def work():
        # stands in for stepping the shard: rank 1 is the slow one
        el = 0.05 + 0.1 * ranks.rank
        time.sleep(el)
        return units, el

    res = shard.timed_shard(ranks, work)
    seen = [None] * world
    ranks.dist.all_gather_object(seen, [m.seed for m in mine])
    np.save(os.path.join(out_dir, f"r{rank}.npy"),
            np.array([res["units"], res["seconds_max"], res["value"], units], dtype=np.float64))
    with open(os.path.join(out_dir, f"seeds{rank}.txt"), "w") as fh:
        fh.write(repr(seen))
    ranks.dist.destroy_process_group()


def test_two_gloo_ranks_shard_the_ensemble(tmp_path):
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    members = synth.ensemble(0)
    total = sum(shard.member_weight(m.nTheta) for m in members)
    res = [np.load(tmp_path / f"r{r}.npy") for r in range(world)]
    for r in res:
        assert r[0] == total                    # units of all ranks
        assert r[1] == pytest.approx(0.15)      # the slowest rank's own time
        assert r[2] == pytest.approx(total / 0.15)
    assert res[0][3] + res[1][3] == total
    seen = [eval((tmp_path / f"seeds{r}.txt").read_text()) for r in range(world)]
    assert seen[0] == seen[1]
    a, b = set(seen[0][0]), set(seen[0][1])
    assert not a & b and a | b == {m.seed for m in members}
