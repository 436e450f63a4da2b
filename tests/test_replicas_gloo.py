"""The multi-GPU replica path on CPU: two gloo ranks (127.0.0.1) aggregate
throughput as all ranks' work over the slowest rank's time, derive distinct
keys, and split a batch so that every item is owned exactly once."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mocat_gb300 import replicas
    value, tmax, total = replicas.aggregate(units=100.0 * (rank + 1), seconds=1.0 + rank)
    start, stop = replicas.split_batch(4097, rank, world)
    key = replicas.replica_key(7, rank)
    np.save(os.path.join(out_dir, f"r{rank}.npy"), np.array([value, tmax, total, start, stop, key[0], key[1]]))
    dist.destroy_process_group()


def test_two_rank_aggregate_and_split(tmp_path):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(tmp_path / "r0.npy")
    r1 = np.load(tmp_path / "r1.npy")
    for r in (r0, r1):
        assert r[0] == 300.0 / 2.0 and r[1] == 2.0 and r[2] == 300.0
    assert (r0[3], r0[4], r1[3], r1[4]) == (0, 2049, 2049, 4097)
    assert tuple(r0[5:]) != tuple(r1[5:])


def test_split_batch_covers_every_item_once():
    from mocat_gb300 import replicas
    for B in (1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            seen = np.zeros(B, int)
            for r in range(world):
                a, b = replicas.split_batch(B, r, world)
                seen[a:b] += 1
            assert (seen == 1).all()


def test_aggregate_without_process_group():
    from mocat_gb300 import replicas
    assert replicas.aggregate(10.0, 2.0) == (5.0, 2.0, 10.0)
