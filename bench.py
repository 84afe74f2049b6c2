#!/usr/bin/env python
"""Benchmark: plain path tracer on the displaced-icosphere workload, 1 GB300.

Workload (one step = one full render): the open-front box of 5 Lambertian walls and a 0.5x0.5
ceiling light (Le 10) holding a level-8 icosphere (1,310,720 triangles) radially displaced by
0.1 * fbm(8 octaves, omega 0.5) with a wrinkled Lambertian texture (8 octaves, omega 0.5);
1024 x 1024 pixels, 64 spp, 8 bounces, Russian roulette from bounce 3, sampler seed 0.
67,108,864 paths per step.  Synthetic seeded data written in the reference's own .scene /
.subject / .bin formats (lighttransportsimulation_gb300.scenes).

Reported (one JSON line on rank 0):
  value      Mpaths/s with the scene and BVH resident in HBM (device time, CUDA events on the
             renderer's stream, max over ranks);
  e2e        Mpaths/s through the public API per step: scene upload from host (H2D), LBVH
             build, render, film read back (D2H);
  roofline   the render kernel's BVH-node + triangle + film bytes (counted by the kernel) per
             launch / launch time, against the measured HBM copy bandwidth;
  lbvh       device time of the bit-exact LBVH build on 1M and 16M random triangles (seed 1)
             against the 304 B/primitive algorithmic model;
  cpu_baseline  the oracle's CPU port of the reference integrator (OpenMP, all host cores) on
             a bounded pixel sample of the same workload.
--impl reference times that CPU port alone, on the same workload and metric.
Inputs (BVH + triangles, ~150 MB) exceed the 129 MB L2, so no flush runs between steps.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="displaced_icosphere_box", width=1024, height=1024, spp=64, max_bounce=8, rr_start=3,
                seed=0, level=8)
SMALL = dict(name="displaced_icosphere_box_small", width=256, height=256, spp=16, max_bounce=8, rr_start=3,
             seed=0, level=6)
# material and divergence stress: glass + 8 rough conductor spheres of 261,120 tris each, marble floor,
# area + infinite light
STRESS = dict(name="stress_glass_conductors", width=1920, height=1080, spp=256, max_bounce=16, rr_start=4,
              seed=0, level=0)


def scene_dir(wl):
    from lighttransportsimulation_gb300 import scenes
    d = os.path.join(tempfile.gettempdir(), f"lts_bench_{wl['name']}_{wl['level']}")
    marker = os.path.join(d, "done")
    if not os.path.exists(marker):
        os.makedirs(d, exist_ok=True)
        if wl is STRESS:
            scenes.write_stress_scene(d)
        else:
            scenes.write_displaced(d, level=wl["level"])
        open(marker, "w").write("ok")
    if wl is STRESS:
        return d, "stress", "stress"
    return d, "box", "displaced"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 2 + k and r[2 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_port_sample(wl, seconds_target=15.0, threads=None):
    """Times the oracle's CPU port of the reference integrator on a pixel band of the workload.
    Returns dict(value=Mpaths/s, cores, sample) or None when the port is not built."""
    exe = os.path.join(ROOT, "oracle", "_build", "lts_port")
    if not os.path.exists(exe):
        return None
    d, sc, sub = scene_dir(wl)
    threads = threads or os.cpu_count()
    # grow the band until the run takes a meaningful time (bounded)
    rows = 8
    while True:
        y0 = wl["height"] // 2 - rows // 2
        out = os.path.join(tempfile.gettempdir(), "lts_port_bench.ltsd")
        cmd = [exe, "render", d + "/", sc, sub, out, wl["width"], wl["height"], wl["spp"], wl["max_bounce"],
               wl["rr_start"], wl["seed"], 0, y0, wl["width"], y0 + rows, threads, 0, 1]
        t0 = time.time()
        subprocess.run([str(c) for c in cmd], check=True, capture_output=True)
        el = time.time() - t0
        from oracle import ltsd
        r = ltsd.read(out)
        secs = float(r["time_s"][0])
        if secs >= seconds_target / 4 or rows >= wl["height"] or el > seconds_target:
            paths = wl["width"] * rows * wl["spp"]
            return {"value": paths / secs / 1e6, "unit": "Mpaths/s", "cores": int(r["threads"][0]), "kind": "port",
                    "sample": f"rows {y0}..{y0 + rows} of {wl['width']}x{wl['height']} at {wl['spp']} spp "
                              f"({paths} paths, {secs:.2f} s)"}
        rows = min(wl["height"], rows * max(2, int(seconds_target / 4 / max(secs, 1e-3)) + 1))


def dist_setup(n):
    """One process per GPU (torchrun's RANK / WORLD_SIZE / LOCAL_RANK / MASTER_*): replicas of the
    same render, no collective on the data path; NCCL on GPUs, gloo without (host-side tests)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return rank, world, local, dist


def barrier_max(dist, value):
    """The largest `value` over the ranks (the timing every replica reports is the slowest's)."""
    if dist is None:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, units_per_rank, seconds_max):
    """Whole-job throughput of `world` replicas each doing `units_per_rank` (weak scaling), over
    the slowest replica's time."""
    return world * units_per_rank / seconds_max


def run_reference(args, wl):
    # CPU arm: rank 0 alone runs; other ranks of a torchrun launch exit without work
    if int(os.environ.get("RANK", "0")) != 0:
        return
    vals = []
    for _ in range(args.warmup):
        cpu_port_sample(wl, seconds_target=4.0)
    t0 = time.time()
    res = None
    for _ in range(args.steps):
        res = cpu_port_sample(wl, seconds_target=8.0)
        if res is None:
            print(json.dumps({"impl": "reference", "unavailable": "oracle CPU port not built (oracle/_build/lts_port)"}))
            return
        vals.append(res["value"])
    el = time.time() - t0
    v = statistics.median(vals)
    line = {"metric": "Mpaths/s", "value": v, "unit": "Mpaths/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * el / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": wl["name"], "width": wl["width"], "height": wl["height"], "spp": wl["spp"],
                       "max_bounce": wl["max_bounce"], "rr_start": wl["rr_start"], "seed": wl["seed"],
                       "triangles": (20 * 4 ** wl["level"] + 12) if wl is not STRESS else 9 * 261120 + 12},
            "cpu_baseline": {**res, "value": v},
            "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def lbvh_bench(ctx, n, steps, warmup, mode, peaks):
    import ctypes

    import numpy as np
    import torch

    from lighttransportsimulation_gb300 import scenes
    tris = torch.from_numpy(scenes.random_triangles(n, seed=1).reshape(-1)).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream())
    torch.cuda.synchronize()
    for _ in range(warmup):
        ctx.check(ctx.lib.lts_bvh_build_device_async(ctx.h, ctypes.c_void_p(tris.data_ptr()), n, mode, -1))
    ctx.check(ctx.lib.lts_bvh_dump_get(ctx.h, None))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ctx.check(ctx.lib.lts_bvh_build_device_async(ctx.h, ctypes.c_void_p(tris.data_ptr()), n, mode, -1))
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    m = ctx.metrics()
    ctx.check(ctx.lib.lts_bvh_dump_get(ctx.h, None))
    m = ctx.metrics()
    stages = [round(x, 4) for x in m.bvh_stage_ms]
    alg = 304.0 * n
    gbs = alg / (ms * 1e-3) / 1e9
    del tris
    torch.cuda.empty_cache()
    return {"n": n, "ms": round(ms, 4), "stage_ms_last": stages, "algorithmic_bytes": alg, "achieved_gbs": round(gbs, 1),
            "frac_of_hbm": round(gbs / peaks["hbm_gbs"], 4)}


MLP_FWD_FLOP = 2 * (96 * 64 + 4 * 64 * 64 + 64 * 3)  # per query: the six layers' products (3 outputs)
MLP_TRAIN_FLOP = MLP_FWD_FLOP + 2 * (3 * 64 + 4 * 64 * 64) + MLP_FWD_FLOP  # + activation and weight gradients


def mlp_bench(ctx, steps, warmup, peaks, queries=1920 * 1080, train_rows=65536):
    """Device time of the radiance-cache network's inference over one film of queries (1920x1080,
    the cache workload's resolution) and of one training step on 65,536 path-suffix samples (the
    per-frame training set), through the device-pointer C-ABI on the context's stream.  Features:
    seeded uniform [-1, 1) bf16 values; targets uniform (0, 1]."""
    import torch

    import lighttransportsimulation_gb300 as lts
    g = torch.Generator(device="cuda").manual_seed(5)
    feat = (torch.rand((queries, 96), generator=g, device="cuda") * 2 - 1).to(torch.bfloat16).view(torch.int16)
    tfeat = feat[:train_rows].contiguous()
    targ = torch.rand((train_rows, 3), generator=g, device="cuda") * 0.999 + 0.001
    out = torch.empty((queries, 3), device="cuda")
    loss = torch.zeros(1, device="cuda")
    net = lts.RadianceCacheMLP(ctx, seed=7)
    stream = torch.cuda.ExternalStream(ctx.stream())
    torch.cuda.synchronize()
    res = {}
    for name, call, rows, flop in (
            ("forward", lambda: net.forward_device_async(feat.data_ptr(), queries, out.data_ptr()), queries,
             MLP_FWD_FLOP),
            ("train", lambda: net.train_step_device_async(tfeat.data_ptr(), targ.data_ptr(), train_rows, 1e-3,
                                                           loss.data_ptr()), train_rows, MLP_TRAIN_FLOP)):
        for _ in range(warmup):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            call()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        tf = rows * flop / (ms * 1e-3) / 1e12
        res[name] = {"rows": rows, "ms": round(ms, 4), "mrows_s": round(rows / (ms * 1e-3) / 1e6, 1),
                     "flop_per_row": flop, "tflops": round(tf, 2), "frac_of_bf16": round(tf / peaks["bf16_tflops"], 4)}
    res["train"]["loss"] = round(float(loss.item()), 6)
    return res


def profiled_traffic(kernel, workload, bvh_width):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (dram__bytes_read.sum +
    dram__bytes_write.sum over every launch of one render, divided by the launches), or None."""
    path = os.path.join(ROOT, "profiles", "trace_wavefront_bench.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        m = re.search(r"<!-- traffic: (.*) -->", line)
        if not m:
            continue
        kv = dict(x.split("=", 1) for x in m.group(1).split())
        if kv.get("kernel") == kernel and kv.get("workload") == workload and kv.get("bvh_width") == str(bvh_width):
            return int(kv["bytes_per_launch"])
    return None


def run_gpu(args, wl):
    import ctypes

    import numpy as np
    import torch

    import lighttransportsimulation_gb300 as lts
    rank, world, local, dist = dist_setup(args.gpus)
    peaks, peak_kind = measured_peaks()
    d, sc, sub = scene_dir(wl)
    ctx = lts.Context(local)
    scene = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
    ctx.set_option("bvh_width", args.bvh_width)
    ctx.set_option("render_bvh", args.render_bvh)
    if args.pool:
        ctx.set_option("wavefront_pool", args.pool)
    integ = lts.PathTracingIntegrator(wl["max_bounce"], wl["rr_start"], scene, integrator=args.integrator)
    desc = integ.desc(wl["spp"], wl["seed"])
    stream = torch.cuda.ExternalStream(ctx.stream())
    paths = wl["width"] * wl["height"] * wl["spp"]

    # warm-up (also builds the LBVH and the leaf-ordered triangles)
    for _ in range(args.warmup):
        ctx.check(ctx.lib.lts_render_async(ctx.h, ctypes.byref(desc)))
    torch.cuda.synchronize()
    ctx.check(ctx.lib.lts_film_get(ctx.h, None, None))

    # device-resident timed region
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kernel_ms = []
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            ctx.check(ctx.lib.lts_render_async(ctx.h, ctypes.byref(desc)))
        e1.record(stream)
        e1.synchronize()
    ctx.check(ctx.lib.lts_film_get(ctx.h, None, None))
    mt = ctx.metrics()
    launches_step, iters_step = mt.render_launches, mt.render_iterations
    ms = e0.elapsed_time(e1) / args.steps
    ms = barrier_max(dist, ms)
    value = replica_throughput(world, paths, ms * 1e-3) / 1e6

    # one counted render for the roofline's algorithmic bytes and the per-stage device times (the
    # same kernels, launched one by one instead of as graphs so that each stage can be timed)
    ctx.set_option("wavefront_graph", 0)
    r = integ.render(wl["spp"], wl["seed"], film=False)
    mr = ctx.metrics()
    render_bvh_ms = round(mr.render_bvh_ms, 3)
    ctx.set_option("wavefront_graph", 1)
    stages = None
    if args.integrator == 0:
        kernel, kernel_ms, kernel_launches = "k_pathtrace", r["render_ms"], 1
        alg_bytes = 64.0 * r["node_visits"] + 48.0 * r["tri_tests"] + 32.0 * paths
        alg_text = "64 B per BVH node visit + 48 B per triangle test + 32 B film per path"
    else:
        names = ["generate", "trace", "finalize", "shade", "compact", "gather"]
        stages = {n: round(mr.render_stage_ms[k], 3) for k, n in enumerate(names)}
        # k_wf_trace (path, shadow and MIS rays in one launch): nodes, triangles, plus the path-state
        # bytes each ray reads and writes
        node_b = 80.0 if args.bvh_width == 8 else 64.0
        state = [56.0, 40.0, 88.0]
        alg_bytes = sum(node_b * mr.kind_node_visits[k] + 48.0 * mr.kind_tri_tests[k] + state[k] * mr.kind_rays[k]
                        for k in range(3))
        alg_text = (f"{int(node_b)} B per BVH node visit + 48 B per triangle test + path state per ray "
                    f"(56 B path ray, 40 B shadow ray, 88 B MIS ray)")
        kernel = "k_wf_trace"
        kernel_ms = mr.render_stage_ms[1]
        kernel_launches = mr.render_iterations
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9
    traffic = profiled_traffic(kernel, wl["name"], args.bvh_width)

    # end to end through the public API: upload scene (H2D), build, render, read film (D2H)
    h2d = scene.info["triangles"] * 48 + scene.info["triangles"] * 16 * 2
    d2h = wl["width"] * wl["height"] * 12
    t_e2e = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
        lts.PathTracingIntegrator(wl["max_bounce"], wl["rr_start"], s2, integrator=args.integrator).render(
            wl["spp"], wl["seed"])
        t_e2e.append(time.perf_counter() - t0)
    e2e_s = barrier_max(dist, statistics.median(t_e2e))
    e2e = replica_throughput(world, paths, e2e_s) / 1e6

    lbvh = None
    if rank == 0 and not args.skip_lbvh:
        lbvh = [lbvh_bench(ctx, n, 5, 3, lts.BVH_SORTED, peaks) for n in (1_000_000, 16_000_000)]
    cpu = cpu_port_sample(wl) if (rank == 0 and world == 1 and not args.skip_cpu) else None
    if rank == 0:
        line = {
            "metric": "Mpaths/s", "value": round(value, 3), "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl["name"], "width": wl["width"], "height": wl["height"], "spp": wl["spp"],
                       "max_bounce": wl["max_bounce"], "rr_start": wl["rr_start"], "seed": wl["seed"],
                       "triangles": scene.info["triangles"],
                       "integrator": ["megakernel", "wavefront"][args.integrator],
                       "bvh": ("sorted-leaf LBVH" if args.bvh_width == 2 else
                               {0: "sorted-leaf LBVH, collapsed 8-wide (greedy)",
                                1: "PLOC tree over the LBVH's Morton order, collapsed 8-wide (SAH-optimal)",
                                2: "PLOC tree over the LBVH's Morton order, collapsed 8-wide (greedy)"}[args.render_bvh]),
                       "path_pool": args.pool or "automatic (all paths of the render, up to 2^26)",
                       "l2": "inputs (BVH + triangles) exceed L2; no flush", "parallelism": f"replicas x{world}"},
            "mrays_per_s": round(r["rays"] / (r["render_ms"] * 1e-3) / 1e6, 2),
            "e2e": {"value": round(e2e, 3), "unit": "Mpaths/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "seconds_per_step": round(e2e_s, 4)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": round(achieved / peaks["hbm_gbs"], 4),
                         "traffic": traffic, "traffic_source": "profiles/trace_wavefront_bench.md" if traffic else None,
                         "kernel": kernel, "launches_per_step": kernel_launches,
                         "kernel_ms_per_step": round(kernel_ms, 3), "peak_kind": peak_kind,
                         "algorithmic": alg_text, "algorithmic_bytes_per_step": alg_bytes},
            "stage_ms": stages,
            "traversal": {"node_visits": r["node_visits"], "tri_tests": r["tri_tests"], "rays": r["rays"],
                          "render_bvh_build_ms": render_bvh_ms,
                          "rays_by_kind": {"path": mr.kind_rays[0], "shadow": mr.kind_rays[1], "mis": mr.kind_rays[2]}},
            "lbvh": lbvh,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": int(args.steps) * launches_step,
            "kernel_launches_per_step": launches_step,
            "wavefront_iterations_per_step": iters_step,
        }
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()


def views64(args):
    """Batched uneven views (the scene of the main workload, 8 bounces): 64 cameras at radius 3.5
    looking at the origin through the box's open front (directions drawn on the cap z >= 0.5 of
    the sphere, seed 4), resolutions drawn from {128^2, 256^2, 512x384, 1024^2}, spp from
    {4, 16, 64}.  Aggregate Mpaths/s of: each view rendered alone; all views batched; batched
    after the autotuner; batched with the radiance cache shared by all views."""
    import numpy as np

    import lighttransportsimulation_gb300 as lts
    wl = WORKLOAD
    rng = np.random.default_rng(4)
    sizes = [(128, 128), (256, 256), (512, 384), (1024, 1024)]
    views = []
    while len(views) < 64:
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        if d[2] < 0.5:
            continue
        w, h = sizes[rng.integers(0, 4)]
        views.append(dict(frm=tuple(float(x) for x in 3.5 * d), at=(0.0, 0.0, 0.0), up=(0, 1, 0), vfov=40.0, focus=3.5,
                          width=w, height=h, spp=int(rng.choice([4, 16, 64])), seed=len(views)))
    paths = sum(v["width"] * v["height"] * v["spp"] for v in views)
    ctx = lts.Context(0)
    d, sc, sub = scene_dir(wl)
    scene = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
    maxb, rr = wl["max_bounce"], wl["rr_start"]
    lts.render_views(scene, views[:2], maxb, rr)  # warm-up: BVH, buffers
    t_alone = sum(lts.render_views(scene, [v], maxb, rr)[1] for v in views)
    _, t_batch = lts.render_views(scene, views, maxb, rr)
    tuned = lts.autotune_views(scene, views, maxb, rr)
    _, t_tuned = lts.render_views(scene, views, maxb, rr)
    lts.RadianceCacheMLP(ctx, seed=7)
    ctx.set_option("radiance_cache", 1)
    biases = []
    for _ in range(12):  # the cache trains on each render; the last render is the timed one
        _, t_cached = lts.render_views(scene, views, maxb, rr)
        biases.append(round(ctx.metrics().cache_bias, 4))
    m = ctx.metrics()
    ctx.set_option("radiance_cache", 0)
    line = {"metric": "Mpaths/s", "unit": "Mpaths/s", "higher_is_better": True, "data": "synthetic",
            "config": {"workload": "64_uneven_views_displaced_icosphere_box", "views": 64, "paths": paths,
                       "max_bounce": maxb, "rr_start": rr,
                       "sizes": {f"{w}x{h}": sum(1 for v in views if (v["width"], v["height"]) == (w, h))
                                 for w, h in sizes},
                       "spp": {str(k): sum(1 for v in views if v["spp"] == k) for k in (4, 16, 64)}},
            "one_by_one": round(paths / (t_alone * 1e-3) / 1e6, 2),
            "batched": round(paths / (t_batch * 1e-3) / 1e6, 2),
            "batched_autotuned": round(paths / (t_tuned * 1e-3) / 1e6, 2), "autotune": tuned,
            "batched_autotuned_cached": round(paths / (t_cached * 1e-3) / 1e6, 2),
            "cache": {"bias": round(m.cache_bias, 4), "bias_by_render": biases, "train_samples": m.cache_train_samples,
                      "train_ms": round(m.cache_train_ms, 3)},
            "ms": {"one_by_one": round(t_alone, 2), "batched": round(t_batch, 2), "autotuned": round(t_tuned, 2),
                   "cached": round(t_cached, 2)}}
    print(json.dumps(line))
    ctx.close()


TTR_LEVELS = (0.05, 0.03, 0.02, 0.015, 0.0125, 0.01)


def time_to_rmse(args):
    """Time for the cached wavefront renderer and for the plain megakernel to bring the stress scene
    (1920x1080, 16 bounces, roulette from 4) to an RMSE <= target against an FP64 oracle render.
    The oracle is the FP64 megakernel on a centred crop at high spp; RMSE is taken over the crop's
    interior (2 pixels in from its edge: border pixels of a crop render miss splats from outside).
    Both renderers accumulate full frames (film_accumulate); time = summed device time of the
    renders (for the cached renderer this includes the bias check and the Adam steps after each
    frame, and its warm-up frames)."""
    import numpy as np

    import lighttransportsimulation_gb300 as lts
    wl = STRESS
    W, H = wl["width"], wl["height"]
    cw, ch = args.ttr_crop
    x0, y0 = (W - cw) // 2, (H - ch) // 2
    x1, y1 = x0 + cw, y0 + ch
    ctx = lts.Context(0)
    d, sc, sub = scene_dir(wl)
    scene = lts.Scene.parse(ctx, d, sc, sub, W, H)
    maxb, rr = wl["max_bounce"], wl["rr_start"]

    def interior(film):
        img = film.reshape(H, W, 3)[::-1]  # the resolve flips rows; undo to index by pixel row
        return img[y0 + 2:y1 - 2, x0 + 2:x1 - 2].astype(np.float64)

    # FP64 oracle on the crop, in passes of at most 256 spp
    t0 = time.time()
    oracle_ms = 0.0
    o = lts.PathTracingIntegrator(maxb, rr, scene, integrator=lts.INTEGRATOR_FP64)
    spp_pass = min(args.ttr_oracle_spp, 256)
    npass = max(1, args.ttr_oracle_spp // spp_pass)
    half = None
    for k in range(npass):
        ctx.set_option("film_accumulate", 0 if k == 0 else 1)
        r = o.render(spp_pass, 50_000 + k, crop=(x0, y0, x1, y1))
        oracle_ms += r["render_ms"]
        if k == npass // 2 - 1:
            half = interior(r["film"])
    oracle = interior(r["film"])
    ctx.set_option("film_accumulate", 0)
    # the oracle's own error, estimated from its first half against the whole
    oracle_err = float(np.sqrt(np.mean((half - oracle) ** 2))) if half is not None else None

    def run(kind):
        integ = lts.PathTracingIntegrator(maxb, rr, scene, integrator=0 if kind == "plain" else 1)
        spp = args.ttr_spp_plain if kind == "plain" else args.ttr_spp_cached
        dev_ms, curve, reached = 0.0, [], None
        if kind == "cached":
            lts.RadianceCacheMLP(ctx, seed=7)
            ctx.set_option("radiance_cache", 1)
            for k in range(args.ttr_warmup):
                ctx.set_option("film_accumulate", 0)
                dev_ms += integ.render(1, 90_000 + k, film=False)["render_ms"]
        frame = 0
        while dev_ms < 1000 * args.ttr_max_seconds:
            ctx.set_option("film_accumulate", 0 if frame == 0 else 1)
            r = integ.render(spp, 1_000 + frame)
            dev_ms += r["render_ms"]
            frame += 1
            e = float(np.sqrt(np.mean((interior(r["film"]) - oracle) ** 2)))
            curve.append((frame * spp, round(dev_ms / 1000, 3), round(e, 5)))
            if e <= args.ttr_target:
                reached = dev_ms / 1000
                break
        m = ctx.metrics()
        ctx.set_option("radiance_cache", 0)
        ctx.set_option("film_accumulate", 0)
        levels = {}
        for lv in TTR_LEVELS:
            hit = next((c for c in curve if c[2] <= lv), None)
            levels[str(lv)] = hit[1] if hit else None
        out = {"seconds_to_target": reached, "seconds_run": round(dev_ms / 1000, 3), "spp": frame * spp,
               "final_rmse": curve[-1][2], "seconds_to_rmse": levels,
               "curve": curve[:: max(1, len(curve) // 12)] + curve[-1:]}
        if kind == "cached":
            out.update(cache_bias=round(m.cache_bias, 4), train_loss=round(m.cache_train_loss, 4),
                       warmup_frames=args.ttr_warmup)
        return out

    plain = run("plain")
    cached = run("cached")
    line = {"metric": "time-to-RMSE", "target_rmse": args.ttr_target, "unit": "s", "higher_is_better": False,
            "config": {"workload": wl["name"], "width": W, "height": H, "max_bounce": maxb, "rr_start": rr,
                       "crop": [x0, y0, x1, y1], "oracle_spp": npass * spp_pass,
                       "oracle_seconds": round(oracle_ms / 1000, 2), "oracle_rmse_estimate": oracle_err,
                       "frame_spp": {"plain": args.ttr_spp_plain, "cached": args.ttr_spp_cached}},
            "plain_megakernel": plain, "cached_wavefront": cached,
            "speedup": (plain["seconds_to_target"] / cached["seconds_to_target"])
            if plain["seconds_to_target"] and cached["seconds_to_target"] else None,
            "speedup_by_rmse": {k: (round(plain["seconds_to_rmse"][k] / v, 2) if v and plain["seconds_to_rmse"][k] else None)
                                for k, v in cached["seconds_to_rmse"].items()},
            "wall_s": round(time.time() - t0, 1)}
    print(json.dumps(line))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--small", action="store_true", help="256x256x16 spp level-6 sphere (quick check)")
    ap.add_argument("--stress", action="store_true",
                    help="the glass + rough-conductor stress scene (1920x1080, 256 spp, 16 bounces)")
    ap.add_argument("--skip-lbvh", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--integrator", type=int, default=1, choices=[0, 1], help="0 megakernel, 1 wavefront")
    ap.add_argument("--bvh-width", type=int, default=8, choices=[2, 8],
                    help="traversal structure: 8-wide compressed BVH or the binary LBVH")
    ap.add_argument("--lbvh-only", type=int, default=0, metavar="N",
                    help="only time the LBVH build over N random triangles (seed 1)")
    ap.add_argument("--render-bvh", type=int, default=1, choices=[0, 1, 2],
                    help="tree the 8-wide BVH is collapsed from: 1 PLOC clustering with the SAH-optimal "
                         "collapse, 2 PLOC with the greedy collapse, 0 the LBVH itself")
    ap.add_argument("--pool", type=int, default=0, metavar="PATHS",
                    help="wavefront path-state pool capacity (0: the renderer's automatic size)")
    ap.add_argument("--views64", action="store_true", help="64 batched uneven views (autotuned, with the cache)")
    ap.add_argument("--mlp-only", action="store_true",
                    help="radiance-cache network alone: inference over 1920x1080 queries, one 65,536-sample training step")
    ap.add_argument("--time-to-rmse", action="store_true",
                    help="time for the cached wavefront and the plain megakernel to reach --ttr-target RMSE")
    ap.add_argument("--ttr-target", type=float, default=1e-2)
    ap.add_argument("--ttr-crop", type=int, nargs=2, default=[192, 108])
    ap.add_argument("--ttr-oracle-spp", type=int, default=16384)
    ap.add_argument("--ttr-spp-plain", type=int, default=8)
    ap.add_argument("--ttr-spp-cached", type=int, default=4)
    ap.add_argument("--ttr-warmup", type=int, default=8)
    ap.add_argument("--ttr-max-seconds", type=float, default=60.0)
    args = ap.parse_args()
    wl = SMALL if args.small else (STRESS if args.stress else WORKLOAD)
    if args.time_to_rmse:
        time_to_rmse(args)
        return
    if args.views64:
        views64(args)
        return
    if args.lbvh_only:
        import lighttransportsimulation_gb300 as lts
        ctx = lts.Context(0)
        print(json.dumps(lbvh_bench(ctx, args.lbvh_only, args.steps, args.warmup, lts.BVH_SORTED, measured_peaks()[0])))
        ctx.close()
        return
    if args.mlp_only:
        import lighttransportsimulation_gb300 as lts
        ctx = lts.Context(0)
        print(json.dumps({"mlp": mlp_bench(ctx, args.steps, args.warmup, measured_peaks()[0])}))
        ctx.close()
        return
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_gpu(args, wl)


if __name__ == "__main__":
    main()
