"""The N>1 host path on CPU with the gloo backend: scenes of a batch are split across
ranks with no data exchange, each rank advances its share (CPU oracle here), and the
timing is reduced with a max over ranks, as bench.py does on GPUs."""
import os
import socket
import sys

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n_scenes, out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    import oracle_lib
    from non_ficks_diffusion_gb300 import workloads
    mine = workloads.shard_scenes(n_scenes, world, rank)
    moved = 0.0
    for s in mine:
        desc, parts = workloads.ball_scene(n=16, radius=0.1, center=(0.5, 0.3 + 0.05 * s, 0.5), seed=s)
        o = oracle_lib.oracle_from_desc(desc, parts, precision=0, threads=1)
        t = o.run(2, 1e-4)
        moved += float(np.abs(o.particles()["X"] - parts["X"]).sum()) + 0 * t
    ids = [torch.zeros(n_scenes, dtype=torch.int64) for _ in range(world)]
    mask = torch.zeros(n_scenes, dtype=torch.int64)
    mask[mine] = 1
    dist.all_gather(ids, mask)
    tmax = torch.tensor([float(len(mine))])
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((torch.stack(ids).numpy(), float(tmax.item()), moved))
    dist.barrier()
    dist.destroy_process_group()


def test_scene_sharding_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    n_scenes = 5
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_scenes, q)) for r in range(2)]
    for p in procs:
        p.start()
    masks, tmax, moved = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert (masks.sum(0) == 1).all()          # every scene on exactly one rank
    assert tmax == 3.0 and moved > 0


def test_shard_ranges():
    from non_ficks_diffusion_gb300 import workloads
    for n in (1, 5, 64):
        for w in (1, 2, 3, 8):
            got = sum((workloads.shard_scenes(n, w, r) for r in range(w)), [])
            assert got == list(range(n))
