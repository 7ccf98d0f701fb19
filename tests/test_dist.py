"""The multi-rank bench path on CPU: two gloo ranks, launched as torchrun
would (RANK / WORLD_SIZE / MASTER_* in the environment). Each rank counts its
own independently seeded catalogue (weak scaling, no data-path collective);
the job's time is the slowest rank's and its throughput the sum of all
ranks' triangles over that time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # Each rank's catalogue: the same process, its own seed.
        p, box, edges, _ = bench.workload("box_uniform", rank)
        t_max = bench.barrier_max(10.0 * (rank + 1), world)
        n_sum = bench.barrier_sum(float(rank + 1), world)
        bench.barrier(world)
        out[rank] = (t_max, n_sum, float(p[:, :3].sum()), len(p), box, len(edges))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_time_and_units():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
        for pr in procs:
            pr.start()
        for pr in procs:
            pr.join(timeout=240)
        assert all(pr.exitcode == 0 for pr in procs), [pr.exitcode for pr in procs]
        res = dict(out)
    assert res[0][0] == res[1][0] == 20.0      # max over ranks
    assert res[0][1] == res[1][1] == 3.0       # sum over ranks
    assert res[0][2] != res[1][2]              # independently seeded catalogues
    assert res[0][3:] == res[1][3:]            # same workload shape on every rank
