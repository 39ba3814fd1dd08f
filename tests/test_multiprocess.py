"""The N>1 path on CPU: two gloo ranks.  The path has no data exchange
(replicas: each rank renders its own frame), so what needs checking is the
host logic — max-over-ranks timing, whole-job throughput — and that replicas
produce identical frames."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle_lib as ol
    from zig_ornament_gb300 import ornament, scenes
    # timings differ per rank; the job time is the slowest rank's
    mine = [100.0 + 50.0 * rank, 130.0 - 20.0 * rank]
    total_ms, total_e2e = bench.reduce_max(mine, dist)
    value = bench.job_throughput(world, 1920 * 1080 * 256, 5, total_ms)
    # every replica renders the same frame bit for bit
    scene = scenes.small_test_scene(32, 24)
    bvh = ornament.Bvh(scene)
    cp = ol.make_params(scene.camera, 32, 24, depth=6, textures_count=bvh.scene_textures_count)
    acc, rng, fb, _ = ol.Oracle().render(bvh, cp, 2, threads=1)
    digest = torch.tensor(np.frombuffer(acc.tobytes(), np.int64).copy()).sum()
    gathered = [torch.zeros_like(digest) for _ in range(world)]
    dist.all_gather(gathered, digest)
    out[rank] = (total_ms, total_e2e, value, [int(g) for g in gathered])
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    r0, r1 = out[0], out[1]
    assert r0[:3] == r1[:3]
    assert r0[0] == 150.0 and r0[1] == 130.0
    assert abs(r0[2] - 2 * 1920 * 1080 * 256 * 5 / 0.150 / 1e6) < 1e-6
    assert len(set(r0[3])) == 1
