"""Several GPUs = replicas: each rank renders its own frame range of the same
image and the benchmark reduces times (max) and counts (sum) over ranks.
Checked here with two gloo ranks on the CPU, each rendering its frames with
the oracle: the summed accumulations equal one render of all the frames,
and bench.py's reduction gives the slowest rank's time and the total work."""
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
W = H = 20
FRAMES = 3


def _paths():
    for p in (ROOT, os.path.join(ROOT, "optix-path-tracer_gb300"), os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)


def _worker(rank, world, port, out_dir):
    _paths()
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle
        import ptgb
        o = oracle.Oracle(ptgb.cornell_c1(W, H))
        acc, st = o.render(W, H, FRAMES, frame0=bench.rank_frame0(rank, FRAMES), rr_depth=3,
                           threads=2)
        t = torch.from_numpy(acc.astype(np.float64))
        dist.all_reduce(t)
        red = bench.reduce_over_ranks(1.0 + rank, 10.0 - rank, st["paths"], st["ext_rays"], "cpu")
        if rank == 0:
            np.save(os.path.join(out_dir, "sum.npy"), t.numpy())
            with open(os.path.join(out_dir, "red.json"), "w") as f:
                json.dump({"reduced": red, "paths0": st["paths"], "rays0": st["ext_rays"]}, f)
        else:
            with open(os.path.join(out_dir, "rank1.json"), "w") as f:
                json.dump({"paths": st["paths"], "rays": st["ext_rays"]}, f)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_replicas(oracle_mod, ptgb_mod, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    summed = np.load(tmp_path / "sum.npy")
    red = json.load(open(tmp_path / "red.json"))
    r1 = json.load(open(tmp_path / "rank1.json"))
    # one render of frames [0, 2 * FRAMES)
    o = oracle_mod.Oracle(ptgb_mod.cornell_c1(W, H))
    whole, st = o.render(W, H, 2 * FRAMES, rr_depth=3, threads=2)
    assert np.all(summed[..., 3] == 2 * FRAMES)
    assert np.allclose(summed[..., :3], whole[..., :3], rtol=1e-5, atol=1e-5)
    dev_s, wall, paths, rays = red["reduced"]
    assert dev_s == 2.0 and wall == 10.0  # the slowest rank's times
    assert paths == red["paths0"] + r1["paths"] == st["paths"]
    assert rays == red["rays0"] + r1["rays"] == st["ext_rays"]
