"""CPU, world_size 2 over gloo: the replica logic bench.py uses for N GPUs
(each rank its own image, a barrier, the max of the ranks' times) with the
oracle standing in for the kernels."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import eff64
    from vmbd_gb300 import geometry, synth
    # each rank: its own seeded image on the same geometry (weak scaling)
    wa = geometry.win2winaux((64, 64), (2, 2), 0.5)
    g = eff64.Geometry(wa.sx, (7, 7), wa.csf, wa.sw, wa.nhop, "valid")
    x = synth.blob_edge_image(wa.sx, seed=rank)
    f = synth.gaussian_psfs(wa.K, (7, 7), seed=100 + rank)
    bench.barrier(world)
    y = eff64.forward(x, f, g, wa.ws.astype(np.float64))
    t_local = 1.0 + rank  # a stand-in time per rank (ms)
    t_max = bench.allreduce_max(t_local, world, torch.device("cpu"))
    q.put((rank, float(y.sum()), t_max))
    dist.destroy_process_group()


def test_two_rank_replicas_over_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=10) for _ in range(world))
    # every rank sees the max of the ranks' times; the images differ per rank
    assert all(r[2] == 2.0 for r in res)
    assert res[0][1] != res[1][1]
