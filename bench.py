#!/usr/bin/env python3
"""Benchmark of the GB300 path tracer.  The default workload is the
2,097,152-triangle heightfield (the third benchmark configuration, the one
the 1.5 G rays/s target is stated on): 1920x1080, 256 spp, fBm terrain with
Torrance-Sparrow / Ashikhmin-Shirley / Oren-Nayar tiles, a 2048x1024 HDR sky
importance-sampled through its 2D CDF, consistent mode (NEE + MIS), max depth
50, Russian roulette after depth 10, seeded synthetic scene.
`--workload spheres` is the random-spheres configuration (1920x1080, 128 spp,
488 spheres, reference mode).

One step = one full render of the workload (all frames) through the C
ABI.  Prints one JSON line (rank 0).  `--impl reference` times the CPU
restatement of the reference's device programs (the reference itself needs
the OptiX 6 SDK and an OpenGL window, neither of which exists here) on a
bounded sample of the same workload with all host threads.

`--workload batch` is the batched multi-scene configuration: 64 seeded
heightfield scenes (1e3..1e6 triangles, 256^2..1024^2, 16..256 spp) in one
pt_batch_render per step, after pt_batch_autotune.

`--workload guide` is the learned-guide configuration: the heightfield in a
closed box lit through a 0.5 % opening, 1920x1080, consistent mode with the
guide trained online; one step = 16 guided frames.  After the timed steps it
compares guided and plain MIS at equal device time against a high-spp FP64
plain render (relMSE, eps 1e-2).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "optix-path-tracer_gb300")
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

WORKLOADS = {
    # name: (generator, width, height, spp, render kwargs, description)
    "spheres": ("random_spheres", 1920, 1080, 128, dict(max_depth=50, rr_depth=10),
                "random spheres: 1920x1080, 128 spp, 488 spheres (ground r=1000, 22x22 grid, "
                "3 large), gradient sky, max depth 50, RR after depth 10"),
    "cornell": ("cornell_c1", 512, 512, 64, dict(max_depth=50, rr_depth=3),
                "Cornell box: 512x512, 64 spp, 8 primitives (6 quads + 2 rotated boxes), "
                "one area light, max depth 50, RR after depth 3"),
    "heightfield": ("heightfield_scene", 1920, 1080, 256, dict(max_depth=50, rr_depth=10, mode=1),
                    "triangle heightfield: 1920x1080, 256 spp, 2,097,152 triangles, "
                    "TS/AS/ON tiles, 2048x1024 HDR sky importance-sampled through its 2D CDF "
                    "(consistent mode: NEE + MIS)"),
}

BATCH_DESC = ("batched multi-scene render: 64 seeded heightfield scenes, triangles log-uniform "
              "over 1e3..1e6 (8.96 M in all), square images of 256/512/1024 px, spp U{16..256} "
              "(4.78 G paths in all), 1024x512 HDR sky importance-sampled (consistent mode), "
              "max depth 50, RR after depth 10; one pt_batch_render (one CUDA-graph launch) "
              "per step")
BATCH_KW = dict(max_depth=50, rr_depth=10, mode=1)
GUIDE_DESC = ("learned-guide form: 2,097,152-triangle heightfield (TS/AS/ON tiles) inside a closed "
              "white Lambertian box lit only through a ceiling opening of 0.5 % of the box area "
              "onto a 2048x1024 HDR sky; 1920x1080, consistent mode (NEE + MIS), max depth 50, "
              "RR after depth 10; MLP 76 -> 4x64 -> 8 vMF lobes + selection, BF16 tensor-core "
              "inference and training (<= 2^19 samples per frame, 12 Adam steps per frame, "
              "lr 1e-2); one step = 16 guided frames")

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "traffic.json")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def rank_frame0(rank, frames_per_rank):
    """Replicas: rank r renders frames [r*F, (r+1)*F) of every image (weak
    scaling, no data-path collective)."""
    return rank * frames_per_rank


def reduce_over_ranks(dev_s, wall, paths, rays, device):
    """(slowest rank's device time, slowest wall time, all ranks' paths,
    all ranks' rays) over the process group; the inputs when it has one rank."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return dev_s, wall, float(paths), float(rays)
    t = torch.tensor([dev_s, wall, float(paths), float(rays)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(mx[1]), float(sm[2]), float(sm[3])


def reduce_images(acc64, device):
    """The replicas' accumulators summed into one image: every rank's FP64
    accumulator (H x W x 4: radiance sums and sample counts of its own
    frames) is gathered on rank 0 and added there in rank order, so the
    image is the same on every run (a fixed order of FP64 additions).
    Returns the sum on rank 0, None on the other ranks; the accumulator
    itself with one rank."""
    import numpy as np
    import torch
    import torch.distributed as dist
    a = np.ascontiguousarray(acc64, dtype=np.float64)
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return a
    t = torch.from_numpy(a).to(device)
    world, rank = dist.get_world_size(), dist.get_rank()
    parts = [torch.empty_like(t) for _ in range(world)] if rank == 0 else None
    dist.gather(t, parts, dst=0)
    if rank != 0:
        return None
    total = parts[0].cpu().numpy().copy()
    for r in range(1, world):
        total += parts[r].cpu().numpy()
    return total


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


SMS, SCHEDULERS_PER_SM = 152, 4


def issue_fraction(tr, ext, shadow, trace_ms, sm_mhz):
    """The trace kernels are bound by instruction issue, not by HBM (their
    BVH and records are served from L1/L2).  Warp instructions per ray come
    from a committed ncu capture (smsp__inst_executed.sum / rays of the
    captured launches, extension and occlusion separately); the rate is the
    warp instructions this run's trace launches must have issued over their
    device time, against 152 SMs x 4 schedulers x one instruction per clock
    at the sampled SM clock (the maximum clock when no sample exists)."""
    i_ext, i_occ = tr.get("warp_inst_per_ext_ray"), tr.get("warp_inst_per_shadow_ray")
    if not i_ext or not i_occ:
        return None
    mhz = sm_mhz or 2070.0
    inst = ext * i_ext + shadow * i_occ
    achieved = inst / (trace_ms / 1e3)
    peak = SMS * SCHEDULERS_PER_SM * mhz * 1e6
    return {"warp_inst_per_s": achieved, "peak_warp_inst_per_s": peak, "frac": achieved / peak,
            "sm_mhz": mhz, "warp_inst_per_ext_ray": i_ext, "warp_inst_per_shadow_ray": i_occ,
            "source": tr.get("_inst_source", "committed ncu capture (profiles/)")}


def cpu_sample(scene, w, h, spp, kw, target_s, threads, max_stride=None):
    """Times the CPU oracle on a strided pixel subset of the workload,
    growing the sample until it takes about target_s seconds."""
    sys.path.insert(0, ORACLE)
    import oracle
    o = oracle.Oracle(scene)
    stride, frames = 4096, 4
    while True:
        acc, st = o.render(w, h, frames, pixel_stride=stride, threads=threads, **kw)
        if st["seconds"] >= target_s or (stride == 1 and frames >= spp):
            break
        grow = max(1.5, min(8.0, target_s / max(st["seconds"], 1e-3)))
        if frames < spp:
            frames = min(spp, int(frames * grow) + 1)
        else:
            stride = max(1, int(stride / grow))
    return st, stride, frames


def batch_cpu_scene(ptgb, items):
    """The scene of the batch whose triangle count is the median: the CPU
    sample of the batched workload."""
    k = sorted(range(len(items)), key=lambda i: items[i][3])[len(items) // 2]
    scene, res, spp, tris = items[k]
    return scene, res, spp, tris, k


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import ptgb
    gen, w, h, spp, kw, desc = wl
    if gen == "batch_workload":
        scene, w, spp, tris, k = batch_cpu_scene(ptgb, ptgb.batch_workload())
        h = w
        desc = desc + f" (CPU sample: scene {k}, {tris} triangles, {w}x{h})"
    else:
        scene = getattr(ptgb, gen)(w, h)
    threads = os.cpu_count()
    sys.path.insert(0, ORACLE)
    import oracle
    o = oracle.Oracle(scene)
    # size one step to about 3 s of CPU work
    st, stride, frames = cpu_sample(scene, w, h, spp, kw, 3.0, threads)
    for _ in range(args.warmup):
        o.render(w, h, frames, pixel_stride=stride, threads=threads, **kw)
    secs, paths, rays = 0.0, 0, 0
    for _ in range(args.steps):
        _, s = o.render(w, h, frames, pixel_stride=stride, threads=threads, **kw)
        secs += s["seconds"]
        paths += s["paths"]
        rays += s["ext_rays"] + s["shadow_rays"]
    value = paths / secs
    sample = f"every {stride}th pixel x {frames} of {spp} spp per step ({paths // args.steps} paths)"
    line = {
        "impl": "reference", "metric": "paths/s", "value": value, "unit": "paths/s",
        "mrays_per_s": rays / secs / 1e6, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": desc, "sample": sample},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "OptiX 6 + OpenGL reference cannot run here; CPU restatement of its device "
                "programs (oracle/oracle.cpp) on all host threads",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, wl):
    import numpy as np
    import torch
    import ptgb

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    gen, w, h, spp, kw, desc = wl
    scene = getattr(ptgb, gen)(w, h)
    # per-rank frames: rank r renders frames [r*spp, (r+1)*spp): weak scaling
    frame0 = rank_frame0(rank, spp)
    rend = ptgb.GpuRenderer(scene, device=local, timing=True)
    prm = ptgb.GpuRenderer.params(w, h, spp, frame0=frame0, **kw)
    acc = torch.zeros((h, w, 4), dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        rend.render(prm, acc.data_ptr())
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    dev_ms, paths, ext, shadow, stage = 0.0, 0, 0, 0, [0.0] * 5
    launches, iters = 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()                      # evict L2 between steps
        torch.cuda.synchronize()
        rend.render(prm, acc.data_ptr())   # synchronous; device-timed inside
        st = rend.stats()
        dev_ms += st["render_ms"]
        paths += st["paths"]
        ext += st["ext_rays"]
        shadow += st["shadow_rays"]
        launches += st["kernel_launches"]
        iters += st["iterations"]
        stage = [a + b for a, b in zip(stage, st["stage_ms"])]
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_s = dev_ms / 1e3
    dev_s, wall, tot_paths, tot_rays = reduce_over_ranks(dev_s, wall, paths, ext + shadow,
                                                         f"cuda:{local}")
    value = tot_paths / dev_s

    # ---- end to end through the C ABI with host buffers: upload + BVH build
    # (pt_commit) and render into pinned host memory with the D2H read, on a
    # context with the default options (no per-stage events)
    host_acc = torch.zeros((h, w, 4), dtype=torch.float32).pin_memory()
    host_np = host_acc.numpy()
    rend_e = ptgb.GpuRenderer(scene, device=local)
    rend_e.render(prm, host_np)            # warm-up (graph capture)
    lib = rend_e.lib
    e2e_paths, e2e_t = 0, 0.0
    for i in range(args.steps):
        barrier()
        t1 = time.perf_counter()
        rend_e._c(lib.pt_commit(rend_e.ctx))
        rend_e.render(prm, host_np)
        e2e_t += time.perf_counter() - t1
        e2e_paths += rend_e.stats()["paths"]
    st = rend_e.stats()
    rend_e.close()
    h2d = int(st["upload_bytes"])   # primitive records, transforms and scene tables
    d2h = w * h * 16

    # ---- algorithmic bytes per ray from a counters pass (outside the timing)
    cnt = ptgb.GpuRenderer(scene, device=local, counters=True)
    cprm = ptgb.GpuRenderer.params(w, h, max(1, spp // 16), frame0=frame0, **kw)
    cnt.render(cprm, acc.data_ptr())
    cs = cnt.stats()
    rays_c = cs["ext_rays"] + cs["shadow_rays"]
    n_node = cs["node_fetches"] / rays_c
    n_prim = cs["prim_tests"] / rays_c
    b_ray = 32 + 16 + 80 * n_node + 48 * n_prim
    cnt.close()
    trace_ms = stage[1] + stage[3]
    trace_launches = 2 * iters
    achieved = (ext + shadow) * b_ray / (trace_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic, issue = None, None
    try:
        with open(PROFILE_TRAFFIC) as f:
            tr = json.load(f).get(args.workload)
        if tr:
            traffic = tr["dram_bytes_per_ray"] * (ext + shadow) / trace_launches
            issue = issue_fraction(tr, ext, shadow, trace_ms, None)
    except (OSError, ValueError, KeyError):
        pass

    if issue is not None and clk:
        issue = issue_fraction(tr, ext, shadow, trace_ms, clk.get("sm_mhz"))

    # ---- the replicas' image: each rank's frames in FP64, summed in rank
    # order on rank 0 (outside the timed region)
    image = None
    if world > 1:
        acc64 = torch.zeros((h, w, 4), dtype=torch.float64, device=f"cuda:{local}")
        rend.render64(prm, acc64.data_ptr())
        torch.cuda.synchronize()
        t_red = time.perf_counter()
        total = reduce_images(acc64.cpu().numpy(), f"cuda:{local}")
        t_red = time.perf_counter() - t_red
        if rank == 0:
            image = {"frames": int(total[..., 3].max()), "mean_rgb": [float(x) for x in
                     (total[..., :3].sum(axis=(0, 1)) / total[..., 3].sum())],
                     "reduce_ms": 1e3 * t_red,
                     "order": "FP64 accumulators gathered on rank 0, added in rank order"}

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count()
        cst, stride, frames = cpu_sample(scene, w, h, spp, kw, args.cpu_seconds, threads)
        cpu = {"value": cst["paths"] / cst["seconds"], "unit": "paths/s", "cores": threads,
               "kind": "port",
               "sample": f"every {stride}th pixel x {frames} spp of the same workload "
                         f"({cst['paths']} paths, {cst['seconds']:.1f} s)",
               "mrays_per_s": (cst["ext_rays"] + cst["shadow_rays"]) / cst["seconds"] / 1e6}

    if rank == 0:
        line = {
            "metric": "paths/s", "value": value, "unit": "paths/s",
            "mrays_per_s": tot_rays / dev_s / 1e6,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "frames_per_rank": spp,
                       "l2": "flushed between steps (256 MiB write); per-step working set "
                             "(path state + per-path results) exceeds L2",
                       "parallelism": f"replicas{world}" if world > 1 else "single"},
            "e2e": {"value": e2e_paths / e2e_t, "unit": "paths/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "includes": "pt_commit (scene upload + BVH8 build) + pt_render into pinned "
                                "host memory"},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_trace + k_trace_shadow (BVH8 closest hit)",
                         "peak_source": peak_kind,
                         "bytes_per_ray": b_ray, "nodes_per_ray": n_node,
                         "prims_per_ray": n_prim,
                         "avg_launch_ms": trace_ms / trace_launches,
                         "rays_per_launch": (ext + shadow) / trace_launches,
                         "issue": issue},
            "stage_ms_per_step": {k: v / args.steps for k, v in
                                  zip(["generate", "trace", "shade", "shadow_trace", "finish"],
                                      stage)},
            "wall_s": wall,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        if image is not None:
            line["image"] = image
        print(json.dumps(line), flush=True)
    rend.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batch(args):
    import numpy as np
    import torch
    import ptgb

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    items = ptgb.batch_workload()
    kw = BATCH_KW
    rends = [ptgb.GpuRenderer(sc, device=local) for sc, *_ in items]
    # replicas: rank r renders frames [r*spp, (r+1)*spp) of every scene
    params = [ptgb.GpuRenderer.params(res, res, spp, frame0=rank_frame0(rank, spp), **kw)
              for _, res, spp, _ in items]
    npix = [res * res for _, res, _, _ in items]
    acc = torch.zeros((sum(npix), 4), dtype=torch.float32, device=f"cuda:{local}")
    offs = np.concatenate([[0], np.cumsum(npix)[:-1]]).astype(np.int64)
    jobs = [(r, p, acc.data_ptr() + 16 * int(o)) for r, p, o in zip(rends, params, offs)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    b = ptgb.Batch(device=local)
    t_tune = time.perf_counter()
    tune = b.autotune(jobs)
    t_tune = time.perf_counter() - t_tune

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        b.render(jobs)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    dev_ms, paths, rays, launches, graphs = 0.0, 0, 0, 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()                      # evict L2 between steps
        torch.cuda.synchronize()
        b.render(jobs)                     # synchronous; device-timed inside
        st = b.stats()
        dev_ms += st["render_ms"]
        paths += st["paths"]
        rays += st["ext_rays"] + st["shadow_rays"]
        launches += st["kernel_launches"]
        graphs += st["graph_launches"]
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_s = dev_ms / 1e3
    dev_s, wall, tot_paths, tot_rays = reduce_over_ranks(dev_s, wall, paths, rays,
                                                         f"cuda:{local}")
    value = tot_paths / dev_s

    # ---- the same scenes one at a time (same batch object and tune)
    single_ms = 0.0
    for j in jobs:
        b.render([j])
        single_ms += b.stats()["render_ms"]
    single_value = (paths / args.steps) / (single_ms / 1e3)

    # ---- stage split (host loop with events) and bytes per ray (counters),
    # each on a 1/8-spp copy of the batch
    small = [(r, ptgb.GpuRenderer.params(p.width, p.height, max(1, p.spp // 8),
                                         frame0=p.frame0, **kw), a) for r, p, a in jobs]
    bt = ptgb.Batch(device=local, timing=True)
    bt.set_tune(tune["path_slots"], tune["trace_block"], tune["shade_block"], tune["bvh_width"])
    bt.render(small)
    sst = bt.stats()
    bt.close()
    bc = ptgb.Batch(device=local, counters=True)
    bc.set_tune(tune["path_slots"], tune["trace_block"], tune["shade_block"], tune["bvh_width"])
    bc.render(small)
    cs = bc.stats()
    bc.close()
    rays_c = cs["ext_rays"] + cs["shadow_rays"]
    n_node = cs["node_fetches"] / rays_c
    n_prim = cs["prim_tests"] / rays_c
    b_ray = 32 + 16 + 80 * n_node + 48 * n_prim
    trace_ms = sst["stage_ms"][1] + sst["stage_ms"][3]
    trace_launches = 2 * sst["iterations"]
    rays_t = sst["ext_rays"] + sst["shadow_rays"]
    achieved = rays_t * b_ray / (trace_ms / 1e3) / 1e9
    peak, peak_kind = peaks()

    # ---- end to end: commit every scene (upload + BVH build) and render the
    # batch into pinned host accumulators
    host = [torch.zeros((p.height, p.width, 4), dtype=torch.float32).pin_memory().numpy()
            for p in params]
    hjobs = [(r, p, a) for r, p, a in zip(rends, params, host)]
    e2e_t, e2e_paths = 0.0, 0
    for _ in range(max(1, args.steps // 2)):
        barrier()
        t1 = time.perf_counter()
        for r in rends:
            r._c(r.lib.pt_commit(r.ctx))
        b.render(hjobs)
        e2e_t += time.perf_counter() - t1
        e2e_paths += b.stats()["paths"]
    h2d = sum(int(r.stats()["upload_bytes"]) for r in rends)
    d2h = 16 * sum(npix)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        scene, res, spp, tris, k = batch_cpu_scene(ptgb, items)
        cst, stride, frames = cpu_sample(scene, res, res, spp, kw, args.cpu_seconds,
                                         os.cpu_count())
        cpu = {"value": cst["paths"] / cst["seconds"], "unit": "paths/s",
               "cores": os.cpu_count(), "kind": "port",
               "sample": f"scene {k} of the batch (median size: {tris} triangles, {res}x{res}): "
                         f"every {stride}th pixel x {frames} spp ({cst['paths']} paths, "
                         f"{cst['seconds']:.1f} s)",
               "mrays_per_s": (cst["ext_rays"] + cst["shadow_rays"]) / cst["seconds"] / 1e6}

    if rank == 0:
        line = {
            "metric": "paths/s", "value": value, "unit": "paths/s",
            "mrays_per_s": tot_rays / dev_s / 1e6,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": BATCH_DESC, "scenes": len(items),
                       "paths_per_rank_step": paths // args.steps,
                       "l2": "flushed between steps (256 MiB write); per-step working set "
                             "(8.96 M triangles of geometry, path state, results) exceeds L2",
                       "tune": tune, "autotune_s": t_tune,
                       "parallelism": f"replicas{world}" if world > 1 else "single"},
            "unbatched": {"value": single_value, "unit": "paths/s",
                          "note": "the same 64 scenes rendered one at a time (one graph launch "
                                  "each), device time"},
            "e2e": {"value": e2e_paths / e2e_t, "unit": "paths/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "includes": "pt_commit of all 64 scenes (upload + BVH8 build) + "
                                "pt_batch_render into pinned host accumulators"},
            "gpu_launches": launches,
            "graph_launches": graphs,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "k_trace + k_trace_shadow (BVH8 closest hit, batch)",
                         "peak_source": peak_kind, "bytes_per_ray": b_ray,
                         "nodes_per_ray": n_node, "prims_per_ray": n_prim,
                         "avg_launch_ms": trace_ms / trace_launches,
                         "rays_per_launch": rays_t / trace_launches,
                         "measured_on": "1/8-spp copy of the batch (host loop with events)"},
            "stage_ms_share": {k: v / max(sum(sst["stage_ms"]), 1e-9) for k, v in
                               zip(["generate", "trace", "shade", "shadow_trace", "finish"],
                                   sst["stage_ms"])},
            "wall_s": wall,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    b.close()
    for r in rends:
        r.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_guide(args):
    import numpy as np
    import torch
    import ptgb

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    W, H = 1920, 1080
    kw = dict(max_depth=50, rr_depth=10, mode=1)
    scene = ptgb.guide_box_scene(W, H)
    P = ptgb.GpuRenderer.params
    g = ptgb.GpuRenderer(scene, device=local)
    g.guide_init(1)
    acc = torch.zeros((H, W, 4), dtype=torch.float64, device=f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    spp_step = 16
    base = rank * 100000
    frame = 0
    for _ in range(args.warmup):
        g.render64(P(W, H, spp_step, frame0=base + frame, guide=1, **kw), acc.data_ptr())
        frame += spp_step
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    dev_ms, paths, rays, launches = 0.0, 0, 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        g.render64(P(W, H, spp_step, frame0=base + frame, guide=1, **kw), acc.data_ptr())
        frame += spp_step
        st = g.stats()
        dev_ms += st["render_ms"]
        paths += st["paths"]
        rays += st["ext_rays"] + st["shadow_rays"]
        launches += st["kernel_launches"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    value = paths / (dev_ms / 1e3)

    # ---- equal-time study (rank 0): plain and guided (fresh guide) against
    # an FP64 plain reference of --ref-spp frames
    study = None
    if rank == 0:
        ref_r = ptgb.GpuRenderer(scene, device=local)
        t_ref = time.perf_counter()
        ref = ref_r.render64(P(W, H, args.ref_spp, frame0=1 << 24, **kw)) / args.ref_spp
        t_ref = time.perf_counter() - t_ref
        curves = {}
        for guide in (0, 1):
            r = ref_r if guide == 0 else ptgb.GpuRenderer(scene, device=local)
            if guide:
                r.guide_init(1)
            a = np.zeros((H, W, 4))
            done, tt, pts = 0, 0.0, []
            for chunk in (4, 4, 8, 16, 32, 64, 128, 256, 512):
                img = r.render64(P(W, H, chunk, frame0=done, guide=guide, **kw))
                tt += r.stats()["render_ms"]
                a[..., :3] += img[..., :3]
                done += chunk
                pts.append((tt, ptgb.rel_mse(a / done, ref), done))
            curves[guide] = pts
            if guide:
                r.close()
        ref_r.close()
        gt = np.array([p[0] for p in curves[1]])
        ge = np.array([p[1] for p in curves[1]])

        def guided_time(e):
            if ge.min() <= e <= ge.max():
                return float(np.exp(np.interp(np.log(e), np.log(ge[::-1]), np.log(gt[::-1]))))
            if e < ge.min():  # extrapolate along relMSE ~ 1/time from the last point
                return float(gt[-1] * ge[-1] / e)
            return None

        # the ratio at every plain budget from 128 spp on (the guide's online
        # training is paid back over more frames at larger budgets)
        ratios = {}
        for t, e, n in curves[0]:
            tg = guided_time(e) if n >= 128 else None
            if tg is not None:
                ratios[str(n)] = round(tg / t, 3)
        t_plain, e_plain, spp_plain = curves[0][-1]
        t_guided = guided_time(e_plain)
        study = {"reference": f"plain consistent render, {args.ref_spp} spp, FP64 sums "
                              f"({t_ref:.0f} s); the configuration names 16384 spp",
                 "relmse_eps": 1e-2,
                 "plain": [{"ms": round(t, 1), "relmse": e, "spp": n} for t, e, n in curves[0]],
                 "guided": [{"ms": round(t, 1), "relmse": e, "spp": n} for t, e, n in curves[1]],
                 "plain_final_relmse": e_plain,
                 "guided_time_to_plain_final_ms": t_guided,
                 "plain_time_ms": t_plain,
                 "plain_budget_spp": spp_plain,
                 "time_ratio": t_guided / t_plain,
                 "time_ratio_by_plain_spp": ratios}

    if rank == 0:
        line = {
            "metric": "paths/s", "value": value, "unit": "paths/s",
            "mrays_per_s": rays / (dev_ms / 1e3) / 1e6, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (MLP bf16, fp32 accumulation)",
            "data": "synthetic",
            "config": {"workload": GUIDE_DESC, "frames_per_step": spp_step,
                       "l2": "flushed between steps (256 MiB write); per-step working set exceeds L2",
                       "parallelism": f"replicas{world}" if world > 1 else "single"},
            "e2e": None, "gpu_launches": launches, "roofline": None, "cpu_baseline": None,
            "equal_time": study, "wall_s": wall, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    g.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 5; 2 for the batch workload)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="heightfield", choices=sorted(WORKLOADS) + ["batch", "guide"])
    ap.add_argument("--ref-spp", type=int, default=4096,
                    help="guide workload: spp of the FP64 plain reference")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--spp", type=int, default=0, help="override spp (small profiling cases)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 2 if args.workload == "batch" else 5
    if args.workload == "guide":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the learned guide has no "
                              "counterpart in the reference (plain MIS is its own arm: "
                              "--workload heightfield)"}), flush=True)
        else:
            run_guide(args)
        return
    if args.workload == "batch":
        if args.impl == "reference":
            run_reference(args, ("batch_workload", 0, 0, 0, BATCH_KW, BATCH_DESC))
        else:
            run_batch(args)
        return
    wl = WORKLOADS[args.workload]
    if args.spp:
        wl = wl[:3] + (args.spp,) + wl[4:5] + (wl[5].replace(f"{wl[3]} spp", f"{args.spp} spp"),)
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
