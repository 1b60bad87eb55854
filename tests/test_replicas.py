"""Several GPUs = replicas: each rank renders its own frame range of the same
image; the benchmark reduces times (max) and counts (sum) over ranks and sums
the ranks' images.  Checked here with two gloo ranks on the CPU, each
rendering its frames with the oracle: the image the ranks reduce (FP64
accumulators gathered on rank 0, added in rank order) equals, bit for bit,
the same frames rendered in one process and added in the same order, whose
counts are those of one render of all the frames and whose radiance agrees
with it to float precision; bench.py's reduction gives the slowest rank's
time and the total work."""
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


def rank_image(oracle, scene, rank):
    """FP64 accumulator of one rank's frames (frame order), y-flipped like
    the renderer's accumulators: sums of per-path colours and counts."""
    import bench
    o = oracle.Oracle(scene)
    acc = np.zeros((H, W, 4), np.float64)
    f0 = bench.rank_frame0(rank, FRAMES)
    for f in range(f0, f0 + FRAMES):
        rgb = o.render_paths(W, H, f, np.arange(W * H), rr_depth=3, threads=2)
        acc[..., :3] += rgb.reshape(H, W, 3)[::-1].astype(np.float64)
        acc[..., 3] += 1.0
    return acc


def _worker(rank, world, port, out_dir):
    _paths()
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle
        import ptgb
        scene = ptgb.cornell_c1(W, H)
        acc = rank_image(oracle, scene, rank)
        o = oracle.Oracle(scene)
        _, st = o.render(W, H, FRAMES, frame0=bench.rank_frame0(rank, FRAMES), rr_depth=3,
                         threads=2)
        total = bench.reduce_images(acc, "cpu")
        red = bench.reduce_over_ranks(1.0 + rank, 10.0 - rank, st["paths"], st["ext_rays"], "cpu")
        if rank == 0:
            np.save(os.path.join(out_dir, "sum.npy"), total)
            with open(os.path.join(out_dir, "red.json"), "w") as f:
                json.dump({"reduced": red, "paths0": st["paths"], "rays0": st["ext_rays"]}, f)
        else:
            assert total is None
            with open(os.path.join(out_dir, "rank1.json"), "w") as f:
                json.dump({"paths": st["paths"], "rays": st["ext_rays"]}, f)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_replicas(oracle_mod, ptgb_mod, tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    summed = np.load(tmp_path / "sum.npy")
    red = json.load(open(tmp_path / "red.json"))
    r1 = json.load(open(tmp_path / "rank1.json"))
    # the same frames in one process, added in rank order: bit for bit
    scene = ptgb_mod.cornell_c1(W, H)
    local = rank_image(oracle_mod, scene, 0)
    local += rank_image(oracle_mod, scene, 1)
    assert np.array_equal(summed, local)
    # against one render of frames [0, 2 * FRAMES)
    o = oracle_mod.Oracle(scene)
    whole, st = o.render(W, H, 2 * FRAMES, rr_depth=3, threads=2)
    assert np.all(summed[..., 3] == 2 * FRAMES)
    assert np.allclose(summed[..., :3], whole[..., :3], rtol=1e-5, atol=1e-5)
    dev_s, wall, paths, rays = red["reduced"]
    assert dev_s == 2.0 and wall == 10.0  # the slowest rank's times
    assert paths == red["paths0"] + r1["paths"] == st["paths"]
    assert rays == red["rays0"] + r1["rays"] == st["ext_rays"]
