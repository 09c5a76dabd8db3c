"""The multi-process path on CPU: two gloo ranks (127.0.0.1) exercise the
replica coordination bench.py uses for runs on several GPUs — scene shards,
barrier, max / sum over ranks, whole-job throughput — and the replica
contract that independent ranks stepping the same input get identical results
with no collective on the data path (stepped here by the CPU oracle)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from sph2s_final_gb300 import replicas


def test_shards_are_disjoint_and_cover():
    for n in (0, 1, 7, 256, 1000):
        for w in (1, 2, 3, 8):
            got = [list(replicas.shard(n, r, w)) for r in range(w)]
            flat = [u for g in got for u in g]
            assert flat == list(range(n))
            sizes = [len(g) for g in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, rk, lr = replicas.world()
        assert (ws, rk, lr) == (world, rank, rank)
        replicas.barrier()
        m = replicas.max_over_ranks(10.0 + rank)
        s = replicas.sum_over_ranks(1.0 + rank)
        # one replica of a small scene per rank, stepped by the CPU oracle
        from oracle import oracle as O
        from sph2s_final_gb300 import scenes
        sc = scenes.small_scene(6)
        ro = O.SSRollout(sc.config, sc.fluid.positions, sc.boundary.positions)
        ro.advance(sc.dt, 3)
        x = ro.state()["x"]
        ro.close()
        units = replicas.sum_over_ranks(sc.fluid.num_particles * 3)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), m=m, s=s, x=x, units=units,
                 shard=np.array(list(replicas.shard(256, rank, world))))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    r0, r1 = (np.load(tmp_path / f"rank{r}.npz") for r in (0, 1))
    assert float(r0["m"]) == float(r1["m"]) == 11.0
    assert float(r0["s"]) == float(r1["s"]) == 3.0
    np.testing.assert_array_equal(r0["x"], r1["x"])  # replicas agree bit for bit
    assert float(r0["units"]) == 2 * 216 * 3
    assert set(r0["shard"]).isdisjoint(set(r1["shard"]))
    assert len(r0["shard"]) + len(r1["shard"]) == 256
    assert replicas.throughput(float(r0["units"]), 2.0) == float(r0["units"]) / 2e-3
