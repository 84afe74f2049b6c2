#!/usr/bin/env python
"""Benchmark: the path tracer on the material-stress scene, 1 GB300.

Workload (one step = one full render): inside the open-front box of Lambertian walls with the
0.5x0.5 ceiling light (Le 10), a displaced glass sphere (UV sphere of 261,120 triangles, IOR 1.5),
eight rough Trowbridge-Reitz conductor spheres (261,120 triangles each, alpha drawn from
U[0.05, 0.5], seed 2, pre-transformed copies), a marble-textured Lambertian floor (8 octaves,
omega 0.5, scale 4) and a constant infinite light of 0.5: 2,350,092 triangles; 1920 x 1080
pixels, 256 spp, 16 bounces, Russian roulette from bounce 4, sampler seed 0.  530,841,600 paths
per step.  Synthetic seeded data written in the reference's own .scene / .subject / .bin formats
(lighttransportsimulation_gb300.scenes).

Reported (one JSON line on rank 0):
  value      Mpaths/s of the wavefront integrator with the scene and BVH resident in HBM (device
             time, CUDA events on the renderer's stream, max over ranks);
  e2e        Mpaths/s through the public API per step: scene parse and upload from host (H2D),
             LBVH build, render-BVH build, render, film read back (D2H);
  roofline   the dominant kernel, k_wf_trace: algorithmic bytes per launch = 32 B per BVH node
             visit + 36 B per triangle test (the fixed traversal model), over its CUDA-event
             launch time, against the measured HBM copy bandwidth; beside it the same bytes
             against an L2 copy bandwidth measured in this run, and 16 FP32 ops per node visit +
             40 per triangle test against the FP32 issue rate at the sampled SM clock;
  time_to_rmse  device seconds for the plain megakernel, the plain wavefront and the wavefront
             with the radiance cache to bring the same scene to RMSE <= 1e-2 against an FP64
             oracle render of a centred crop (film accumulated over frames);
  lbvh       device time of the LBVH build on 1M and 16M random triangles (seed 1), in the
             reference's bit-exact mode and in the sorted-leaf mode, against the 304 B/primitive
             algorithmic model;
  cpu_baseline  the oracle's CPU port of the reference integrator (OpenMP, all host cores) on
             a bounded pixel band of the same workload;
  displaced_icosphere  the same figures (value, e2e) for the displaced-icosphere render
             (1,310,732 triangles, 1024 x 1024, 64 spp, 8 bounces);
  watertight the same render with the watertight triangle test (option "watertight");
  instanced  the stress scene with its conductor spheres as instances of one mesh file, 64 spp:
             Mpaths/s, render-BVH bytes and build time through the two-level BVH and through one
             flat tree;
  bdpt       bidirectional path tracing on a box lit by one triangle (256 x 256, 5 bounces):
             Msamples/s beside the two path tracers, and the RMSE BDPT and the wavefront path
             tracer reach in equal device time against a 16,384-spp render; the same for the box
             lit indirectly (the triangle facing the ceiling) against a 65,536-spp render.
--impl reference times that CPU port alone, on the same workload and metric.
Inputs (BVH + triangles, ~400 MB) exceed the 129 MB L2, so no flush runs between steps.
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


# the same scene on a 480x270 film at 64 spp: small cases for profiler captures
STRESS_SMALL = dict(STRESS, name="stress_glass_conductors_480x270", width=480, height=270, spp=64)
WORKLOADS = {"stress": STRESS, "displaced": WORKLOAD, "small": SMALL, "stress_small": STRESS_SMALL}


def is_stress(wl):
    return wl["level"] == 0


def scene_triangles(wl):
    return (20 * 4 ** wl["level"] + 12) if not is_stress(wl) else 9 * 261120 + 12


def scene_dir(wl):
    from lighttransportsimulation_gb300 import scenes
    d = os.path.join(tempfile.gettempdir(), f"lts_bench_{'stress' if is_stress(wl) else wl['name']}_{wl['level']}")
    marker = os.path.join(d, "done")
    if not os.path.exists(marker):
        os.makedirs(d, exist_ok=True)
        if is_stress(wl):
            scenes.write_stress_scene(d)
        else:
            scenes.write_displaced(d, level=wl["level"])
        open(marker, "w").write("ok")
    if is_stress(wl):
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
                       "triangles": scene_triangles(wl)},
            "cpu_baseline": {**res, "value": v},
            "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def lbvh_bench(ctx, n, steps, warmup, modes, peaks):
    """Device time per LBVH build of n random triangles (seed 1) in each of `modes`
    (lts.BVH_REFERENCE: the reference's bit-exact tree; lts.BVH_SORTED: sorted-leaf tree), CUDA
    events on the context's stream, against the 304 B/primitive algorithmic model."""
    import ctypes

    import torch

    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    tris = torch.from_numpy(scenes.random_triangles(n, seed=1).reshape(-1)).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream())
    torch.cuda.synchronize()
    out = []
    for mode in modes:
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
        ctx.check(ctx.lib.lts_bvh_dump_get(ctx.h, None))
        stages = [round(x, 4) for x in ctx.metrics().bvh_stage_ms]
        alg = 304.0 * n
        gbs = alg / (ms * 1e-3) / 1e9
        out.append({"n": n, "mode": "reference" if mode == lts.BVH_REFERENCE else "sorted", "ms": round(ms, 4),
                    "stage_ms_last": stages, "stages": ["bounds", "morton", "sort", "clear", "tree"],
                    "algorithmic_bytes": alg, "achieved_gbs": round(gbs, 1), "frac_of_hbm": round(gbs / peaks["hbm_gbs"], 4)})
    del tris
    torch.cuda.empty_cache()
    return out


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


def l2_copy_gbs(reps=100):
    """Copy bandwidth of a working set that stays in the 129 MB L2: two 24 MiB buffers copied into
    each other in turn (read + write bytes per copy), CUDA events on torch's stream, best of three
    rounds.  The L2 figure that the traversal's byte model is held against."""
    import torch
    n = 24 << 20
    a = torch.ones(n, dtype=torch.uint8, device="cuda")
    b = torch.empty_like(a)
    for _ in range(10):
        b.copy_(a)
        a.copy_(b)
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            b.copy_(a)
            a.copy_(b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * reps * 2 * n / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    del a, b
    return best


def trace_roofline(mr, peaks, peak_kind, l2_gbs, sm_mhz, sms):
    """Roofline of k_wf_trace over one counted render (metrics `mr` of a kernel-by-kernel render):
    the traversal's fixed model, 32 B per BVH node visit + 36 B per triangle test of algorithmic
    bytes and 16 + 40 FP32 ops, per launch and over the launches' CUDA-event time."""
    nodes, tris = sum(mr.kind_node_visits), sum(mr.kind_tri_tests)
    launches = max(1, mr.render_iterations)
    kernel_ms = mr.render_stage_ms[1]
    alg = 32.0 * nodes + 36.0 * tris
    achieved = alg / (kernel_ms * 1e-3) / 1e9
    ops = 16.0 * nodes + 40.0 * tris
    fp32_peak = sms * 128 * sm_mhz * 1e6  # FP32 lanes per SM x clock
    fp32_frac = ops / (kernel_ms * 1e-3) / fp32_peak
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None, "kernel": "k_wf_trace",
            "peak_kind": peak_kind,
            "algorithmic": "32 B per BVH node visit + 36 B per triangle test (per launch: node visits and "
                           "triangle tests of the launch, counted by the kernel)",
            "algorithmic_bytes_per_launch": round(alg / launches), "launches_per_step": launches,
            "kernel_ms_per_step": round(kernel_ms, 3),
            "l2": {"achieved": round(achieved, 1), "peak": round(l2_gbs, 1), "unit": "GB/s",
                   "frac": round(achieved / l2_gbs, 4), "peak_kind": "L2 copy measured in this run"},
            "fp32_issue": {"ops_per_step": ops, "achieved_tops": round(ops / (kernel_ms * 1e-3) / 1e12, 3),
                           "peak_tops": round(fp32_peak / 1e12, 2), "frac": round(fp32_frac, 4),
                           "model": "16 FP32 ops per node visit + 40 per triangle test; peak = SMs x 128 "
                                    "FP32 lanes x sampled SM clock"}}


def render_timed(ctx, desc, steps, stream):
    """Device milliseconds per render of `steps` back-to-back renders (CUDA events on the
    renderer's stream)."""
    import ctypes

    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ctx.check(ctx.lib.lts_render_async(ctx.h, ctypes.byref(desc)))
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def e2e_render(ctx, wl, integrator, reps):
    """Seconds per end-to-end render through the public API: parse + upload the scene, LBVH,
    render-BVH, render, film read back; median of `reps`.  Returns (seconds, h2d, d2h bytes)."""
    import torch

    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dir(wl)
    t, h2d = [], 0
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
        lts.PathTracingIntegrator(wl["max_bounce"], wl["rr_start"], s2, integrator=integrator).render(
            wl["spp"], wl["seed"])
        t.append(time.perf_counter() - t0)
        h2d = ctx.metrics().scene_upload_bytes
    return statistics.median(t), int(h2d), wl["width"] * wl["height"] * 12


def displaced_extra(args, ctx):
    """The displaced-icosphere render (1024 x 1024, 64 spp, 8 bounces, 1,310,732 triangles):
    device Mpaths/s over 3 renders and end to end through the public API."""
    import torch

    import lighttransportsimulation_gb300 as lts
    wl = WORKLOAD
    d, sc, sub = scene_dir(wl)
    scene = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
    integ = lts.PathTracingIntegrator(wl["max_bounce"], wl["rr_start"], scene, integrator=1)
    desc = integ.desc(wl["spp"], wl["seed"])
    stream = torch.cuda.ExternalStream(ctx.stream())
    render_timed(ctx, desc, 2, stream)
    ms = render_timed(ctx, desc, 3, stream)
    paths = wl["width"] * wl["height"] * wl["spp"]
    e2e_s, h2d, d2h = e2e_render(ctx, wl, 1, 1)
    return {"workload": wl["name"], "width": wl["width"], "height": wl["height"], "spp": wl["spp"],
            "max_bounce": wl["max_bounce"], "rr_start": wl["rr_start"], "triangles": scene.info["triangles"],
            "value": round(paths / (ms * 1e-3) / 1e6, 3), "unit": "Mpaths/s", "ms_per_step": round(ms, 3),
            "e2e": {"value": round(paths / e2e_s / 1e6, 3), "unit": "Mpaths/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h}}


def instanced_extra(args, ctx):
    """The stress scene with its eight conductor spheres as instances of one 261,120-triangle
    unit-sphere file (the loader's `instances` record), 1920 x 1080, 64 spp, 16 bounces: device
    Mpaths/s, render-BVH bytes and build time through the two-level BVH (one tree per prototype
    under a top level) and through one flat tree over all 2,350,092 triangles."""
    import torch

    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    wl = dict(STRESS, spp=64)
    d = os.path.join(tempfile.gettempdir(), "lts_bench_stress_instanced")
    marker = os.path.join(d, "done")
    if not os.path.exists(marker):
        os.makedirs(d, exist_ok=True)
        scenes.write_stress_scene(d, instanced=True)
        open(marker, "w").write("ok")
    scene = lts.Scene.parse(ctx, d, "stress_inst", "stress_inst", wl["width"], wl["height"])
    integ = lts.PathTracingIntegrator(wl["max_bounce"], wl["rr_start"], scene, integrator=1)
    desc = integ.desc(wl["spp"], wl["seed"])
    stream = torch.cuda.ExternalStream(ctx.stream())
    paths = wl["width"] * wl["height"] * wl["spp"]
    out = {"workload": "stress_glass_conductors_instanced", "width": wl["width"], "height": wl["height"],
           "spp": wl["spp"], "max_bounce": wl["max_bounce"], "rr_start": wl["rr_start"],
           "triangles": scene.info["triangles"], "instances": scene.info["instances"],
           "prototypes": scene.info["prototypes"]}
    try:
        for tl, key in ((1, "two_level"), (0, "flat")):
            ctx.set_option("two_level_bvh", tl)
            render_timed(ctx, desc, 1, stream)  # builds this mode's render BVH
            m = ctx.metrics()
            assert m.render_two_level == tl
            bvh_ms, bvh_bytes = m.render_bvh_ms, m.render_bvh_bytes
            ms = render_timed(ctx, desc, 2, stream)
            out[key] = {"value": round(paths / (ms * 1e-3) / 1e6, 3), "unit": "Mpaths/s", "ms_per_step": round(ms, 3),
                        "render_bvh_bytes": int(bvh_bytes), "render_bvh_build_ms": round(bvh_ms, 3)}
    finally:
        ctx.set_option("two_level_bvh", 1)
    return out


BDPT_BOX = dict(width=256, height=256, max_bounce=5, rr_start=3, spp=64, seed=11, ref_spp=16384)


def bdpt_extra(args, ctx):
    """Bidirectional path tracing (LTS_INTEGRATOR_BDPT) on the box + icosphere scene lit by one
    ceiling triangle (Lambertian walls, 256 x 256, 5 bounces): device Msamples/s of BDPT and of
    the two path tracers at 64 spp, and the film RMSE that BDPT and the wavefront path tracer
    reach in the same device time (BDPT's 64 spp), against a 16,384-spp wavefront render."""
    import numpy as np
    import torch

    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    wl = BDPT_BOX
    d = os.path.join(tempfile.gettempdir(), "lts_bench_bdpt_box")
    sc, sub = scenes.write_tri_light_box(d)
    scene = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
    stream = torch.cuda.ExternalStream(ctx.stream())
    px = wl["width"] * wl["height"]

    def integ(kind):
        return lts.PathTracingIntegrator(wl["max_bounce"], wl["rr_start"], scene, integrator=kind)

    def timed(kind, spp, seed):
        desc = integ(kind).desc(spp, seed)
        render_timed(ctx, desc, 1, stream)
        return render_timed(ctx, desc, 2, stream)

    out = {"workload": "box_icosphere_one_triangle_light", "width": wl["width"], "height": wl["height"],
           "max_bounce": wl["max_bounce"], "spp": wl["spp"], "unit": "Msamples/s"}
    ms = {}
    for name, kind in (("bdpt", lts.INTEGRATOR_BDPT), ("megakernel", lts.INTEGRATOR_MEGAKERNEL),
                       ("wavefront", lts.INTEGRATOR_WAVEFRONT)):
        ms[name] = timed(kind, wl["spp"], wl["seed"])
        out[name] = round(px * wl["spp"] / (ms[name] * 1e-3) / 1e6, 3)
    out["value"] = out["bdpt"]
    ref = integ(lts.INTEGRATOR_WAVEFRONT).render(wl["ref_spp"], wl["seed"] + 1)["film"].astype(np.float64)
    spp_pt = max(1, int(round(wl["spp"] * ms["bdpt"] / ms["wavefront"])))
    bd = integ(lts.INTEGRATOR_BDPT).render(wl["spp"], wl["seed"] + 2)["film"].astype(np.float64)
    pt = integ(lts.INTEGRATOR_WAVEFRONT).render(spp_pt, wl["seed"] + 3)["film"].astype(np.float64)
    out["equal_time"] = {"device_ms": round(ms["bdpt"], 3), "bdpt_spp": wl["spp"], "wavefront_spp": spp_pt,
                         "reference_spp": wl["ref_spp"],
                         "rmse_bdpt": float(np.sqrt(np.mean((bd - ref) ** 2))),
                         "rmse_wavefront": float(np.sqrt(np.mean((pt - ref) ** 2))),
                         "mean_bdpt": float(bd.mean()), "mean_reference": float(ref.mean())}
    # the same box lit indirectly: the triangle faces the ceiling, so next-event estimation from
    # the room never reaches its emitting side and the path tracer finds the light only by
    # BSDF-sampled bounces off the ceiling, while BDPT's light subpaths start there
    d2 = os.path.join(tempfile.gettempdir(), "lts_bench_bdpt_box_up")
    sc2, sub2 = scenes.write_tri_light_box(d2, facing_up=True)
    scene = lts.Scene.parse(ctx, d2, sc2, sub2, wl["width"], wl["height"])
    ms_b = timed(lts.INTEGRATOR_BDPT, wl["spp"], wl["seed"])
    ms_w = timed(lts.INTEGRATOR_WAVEFRONT, wl["spp"], wl["seed"])
    ref = integ(lts.INTEGRATOR_WAVEFRONT).render(4 * wl["ref_spp"], wl["seed"] + 1)["film"].astype(np.float64)
    spp_pt = max(1, int(round(wl["spp"] * ms_b / ms_w)))
    bd = integ(lts.INTEGRATOR_BDPT).render(wl["spp"], wl["seed"] + 2)["film"].astype(np.float64)
    pt = integ(lts.INTEGRATOR_WAVEFRONT).render(spp_pt, wl["seed"] + 3)["film"].astype(np.float64)
    out["equal_time_indirect"] = {"device_ms": round(ms_b, 3), "bdpt_spp": wl["spp"], "wavefront_spp": spp_pt,
                                  "reference_spp": 4 * wl["ref_spp"],
                                  "bdpt_msamples_s": round(px * wl["spp"] / (ms_b * 1e-3) / 1e6, 3),
                                  "rmse_bdpt": float(np.sqrt(np.mean((bd - ref) ** 2))),
                                  "rmse_wavefront": float(np.sqrt(np.mean((pt - ref) ** 2))),
                                  "mean_bdpt": float(bd.mean()), "mean_reference": float(ref.mean())}
    return out


def run_gpu(args, wl):
    import ctypes

    import torch

    import lighttransportsimulation_gb300 as lts
    rank, world, local, dist = dist_setup(args.gpus)
    peaks, peak_kind = measured_peaks()
    d, sc, sub = scene_dir(wl)
    ctx = lts.Context(local)
    if args.libm_double is not None:
        ctx.set_option("libm_double", args.libm_double)
    scene = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
    ctx.set_option("bvh_width", args.bvh_width)
    ctx.set_option("render_bvh", args.render_bvh)
    if args.pool:
        ctx.set_option("wavefront_pool", args.pool)
    integ = lts.PathTracingIntegrator(wl["max_bounce"], wl["rr_start"], scene, integrator=args.integrator)
    desc = integ.desc(wl["spp"], wl["seed"])
    stream = torch.cuda.ExternalStream(ctx.stream())
    paths = wl["width"] * wl["height"] * wl["spp"]

    # warm-up (also builds the LBVH, the render BVH and the leaf-ordered triangles)
    for _ in range(args.warmup):
        ctx.check(ctx.lib.lts_render_async(ctx.h, ctypes.byref(desc)))
    torch.cuda.synchronize()
    ctx.check(ctx.lib.lts_film_get(ctx.h, None, None))

    # device-resident timed region
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ms = render_timed(ctx, desc, args.steps, stream)
    ctx.check(ctx.lib.lts_film_get(ctx.h, None, None))
    mt = ctx.metrics()
    launches_step, iters_step = mt.render_launches, mt.render_iterations
    ms = barrier_max(dist, ms)
    value = replica_throughput(world, paths, ms * 1e-3) / 1e6
    clocks = clk.summary()

    # one counted render for the roofline's work counts and the per-stage device times (the same
    # kernels, launched one by one instead of as graphs so that each stage can be timed)
    ctx.set_option("wavefront_graph", 0)
    r = integ.render(wl["spp"], wl["seed"], film=False)
    mr = ctx.metrics()
    render_bvh_ms = round(mr.render_bvh_ms, 3)
    ctx.set_option("wavefront_graph", 1)
    stages, roofline = None, None
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    if args.integrator == 1:
        names = ["generate", "trace", "finalize", "shade", "compact", "gather"]
        stages = {n: round(mr.render_stage_ms[k], 3) for k, n in enumerate(names)}
        roofline = trace_roofline(mr, peaks, peak_kind, l2_copy_gbs(), sm_mhz, sms)

    # the watertight triangle test (the fixed mode of the reference's test) on the same render:
    # device Mpaths/s and the trace stage's time
    watertight = None
    if args.integrator == 1 and not args.skip_watertight:
        ctx.set_option("watertight", 1)
        render_timed(ctx, desc, 1, stream)
        wt_ms = render_timed(ctx, desc, max(1, min(args.steps, 3)), stream)
        ctx.set_option("wavefront_graph", 0)
        integ.render(wl["spp"], wl["seed"], film=False)
        wt_trace = ctx.metrics().render_stage_ms[1]
        ctx.set_option("wavefront_graph", 1)
        ctx.set_option("watertight", 0)
        watertight = {"value": round(paths / (wt_ms * 1e-3) / 1e6, 3), "unit": "Mpaths/s",
                      "ms_per_step": round(wt_ms, 3), "trace_ms_per_step": round(wt_trace, 3),
                      "trace_ms_reference_test": round(mr.render_stage_ms[1], 3)}

    # end to end through the public API: parse + upload (H2D), builds, render, film (D2H)
    e2e_s, h2d, d2h = e2e_render(ctx, wl, args.integrator, max(1, min(args.steps, 3)))
    e2e_s = barrier_max(dist, e2e_s)
    e2e = replica_throughput(world, paths, e2e_s) / 1e6

    solo = rank == 0 and world == 1
    lbvh = None
    if rank == 0 and not args.skip_lbvh:
        lbvh = [x for n in (1_000_000, 16_000_000)
                for x in lbvh_bench(ctx, n, 5, 3, (lts.BVH_REFERENCE, lts.BVH_SORTED), peaks)]
    cpu = cpu_port_sample(wl) if (solo and not args.skip_cpu) else None
    ttr = time_to_rmse(args, ctx) if (solo and wl is STRESS and not args.skip_ttr) else None
    extra = displaced_extra(args, ctx) if (solo and wl is STRESS and not args.skip_displaced) else None
    inst = instanced_extra(args, ctx) if (solo and wl is STRESS and not args.skip_instanced) else None
    bdpt = bdpt_extra(args, ctx) if (solo and wl is STRESS and not args.skip_bdpt) else None
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
            "roofline": roofline,
            "stage_ms": stages,
            "traversal": {"node_visits": r["node_visits"], "tri_tests": r["tri_tests"], "rays": r["rays"],
                          "render_bvh_build_ms": render_bvh_ms,
                          "rays_by_kind": {"path": mr.kind_rays[0], "shadow": mr.kind_rays[1], "mis": mr.kind_rays[2]}},
            "watertight": watertight,
            "time_to_rmse": ttr,
            "lbvh": lbvh,
            "cpu_baseline": cpu,
            "displaced_icosphere": extra,
            "instanced": inst,
            "bdpt": bdpt,
            "clocks": clocks,
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
    films_plain, t_batch = lts.render_views(scene, views, maxb, rr)
    tuned = lts.autotune_views(scene, views, maxb, rr)
    _, t_tuned = lts.render_views(scene, views, maxb, rr)
    lts.RadianceCacheMLP(ctx, seed=7)
    ctx.set_option("radiance_cache", 1)
    biases = []
    for _ in range(12):  # the cache trains on each render; the last render is the timed one
        films_cached, t_cached = lts.render_views(scene, views, maxb, rr)
        biases.append(round(ctx.metrics().cache_bias, 4))
    m = ctx.metrics()
    ctx.set_option("radiance_cache", 0)
    # per-view RMSE against the FP64 renderer: each view's camera in a scene file of its own, the
    # FP64 renderer on a centred 32 x 32 crop at args.views_oracle_spp; RMSE over the crop's
    # interior (2 pixels in), for the plain and the cached batched films
    from lighttransportsimulation_gb300 import scenes
    rmse_plain, rmse_cached, oracle_ms = [], [], 0.0
    for k, v in enumerate(views):
        W, H = v["width"], v["height"]
        x0, y0 = (W - 32) // 2, (H - 32) // 2
        name = scenes.with_camera(d, sc, v, f"view64_{k}")
        sv = lts.Scene.parse(ctx, d, name, sub, W, H)
        o = lts.PathTracingIntegrator(maxb, rr, sv, integrator=lts.INTEGRATOR_FP64)
        npass = max(1, args.views_oracle_spp // 256)
        for p in range(npass):
            ctx.set_option("film_accumulate", 0 if p == 0 else 1)
            r = o.render(min(256, args.views_oracle_spp), 70_000 + 97 * k + p, crop=(x0, y0, x0 + 32, y0 + 32))
            oracle_ms += r["render_ms"]
        ctx.set_option("film_accumulate", 0)
        ref = r["film"].reshape(H, W, 3)[::-1][y0 + 2:y0 + 30, x0 + 2:x0 + 30].astype(np.float64)
        for films, out in ((films_plain, rmse_plain), (films_cached, rmse_cached)):
            img = films[k][::-1][y0 + 2:y0 + 30, x0 + 2:x0 + 30].astype(np.float64)
            out.append(round(float(np.sqrt(np.mean((img - ref) ** 2))), 5))
    scene = lts.Scene.parse(ctx, d, sc, sub, wl["width"], wl["height"])
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
            "rmse_vs_fp64": {"oracle": f"FP64 renderer, centred 32x32 crop of each view, {args.views_oracle_spp} spp; "
                                       "RMSE over the crop interior (28x28)",
                             "oracle_seconds": round(oracle_ms / 1000, 2),
                             "plain": rmse_plain, "cached": rmse_cached,
                             "plain_mean": round(float(np.mean(rmse_plain)), 5),
                             "cached_mean": round(float(np.mean(rmse_cached)), 5),
                             "by_spp": {str(q): {"plain": round(float(np.mean([e for e, v in zip(rmse_plain, views)
                                                                                if v["spp"] == q])), 5),
                                                 "cached": round(float(np.mean([e for e, v in zip(rmse_cached, views)
                                                                                 if v["spp"] == q])), 5)}
                                        for q in (4, 16, 64)}},
            "ms": {"one_by_one": round(t_alone, 2), "batched": round(t_batch, 2), "autotuned": round(t_tuned, 2),
                   "cached": round(t_cached, 2)}}
    print(json.dumps(line))
    ctx.close()


TTR_LEVELS = (0.05, 0.03, 0.02, 0.015, 0.0125, 0.01)


def time_to_rmse(args, ctx):
    """Device seconds for the plain megakernel, the plain wavefront and the wavefront with the
    radiance cache to bring the stress scene (1920x1080, 16 bounces, roulette from 4) to an RMSE
    <= target against an FP64 oracle render.

    RMSE = sqrt(mean over pixels x RGB of (I - I_oracle)^2) of the resolved linear film, over the
    interior (2 pixels in) of a centred crop: the oracle is the FP64 renderer on that crop at
    high spp (border pixels of a crop render miss splats from outside it).  Every renderer
    renders full frames and accumulates its film across frames (film_accumulate); its time is the
    summed device time of its renders (for the cached renderer including its warm-up frames and
    the bias check and Adam steps after every frame).  `image_bias` is the relative difference
    of the crop interior's mean from the oracle's at the end of the run."""
    import numpy as np

    import lighttransportsimulation_gb300 as lts
    wl = STRESS
    W, H = wl["width"], wl["height"]
    cw, ch = args.ttr_crop
    x0, y0 = (W - cw) // 2, (H - ch) // 2
    x1, y1 = x0 + cw, y0 + ch
    d, sc, sub = scene_dir(wl)
    scene = lts.Scene.parse(ctx, d, sc, sub, W, H)
    maxb, rr = wl["max_bounce"], wl["rr_start"]
    t_start = time.time()

    def interior(film):
        img = film.reshape(H, W, 3)[::-1]  # the resolve flips rows; undo to index by pixel row
        return img[y0 + 2:y1 - 2, x0 + 2:x1 - 2].astype(np.float64)

    # FP64 oracle on the crop, in passes of at most 1024 spp
    oracle_ms = 0.0
    o = lts.PathTracingIntegrator(maxb, rr, scene, integrator=lts.INTEGRATOR_FP64)
    spp_pass = min(args.ttr_oracle_spp, 1024)
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
    # the oracle's own error, estimated from its first half against the whole (the half's error
    # against the truth is ~sqrt(2) x the whole's, and their difference ~ the whole's error)
    oracle_err = float(np.sqrt(np.mean((half - oracle) ** 2))) if half is not None else None
    omean = float(oracle.mean())

    def run(kind):
        integ = lts.PathTracingIntegrator(maxb, rr, scene, integrator=0 if kind == "megakernel" else 1)
        spp = {"megakernel": args.ttr_spp_plain, "wavefront": args.ttr_spp_wavefront,
               "cached": args.ttr_spp_cached}[kind]
        dev_ms, curve, reached = 0.0, [], None
        if kind == "cached":
            lts.RadianceCacheMLP(ctx, seed=7)
            ctx.set_option("radiance_cache", 1)
            for k in range(args.ttr_warmup):
                ctx.set_option("film_accumulate", 0)
                dev_ms += integ.render(1, 90_000 + k, film=False)["render_ms"]
        frame, img = 0, None
        while dev_ms < 1000 * args.ttr_max_seconds:
            ctx.set_option("film_accumulate", 0 if frame == 0 else 1)
            r = integ.render(spp, 1_000 + frame)
            dev_ms += r["render_ms"]
            frame += 1
            img = interior(r["film"])
            e = float(np.sqrt(np.mean((img - oracle) ** 2)))
            curve.append((frame * spp, round(dev_ms / 1000, 4), round(e, 5)))
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
        out = {"seconds_to_target": round(reached, 4) if reached else None, "seconds_run": round(dev_ms / 1000, 3),
               "spp": frame * spp, "frame_spp": spp, "final_rmse": curve[-1][2],
               "image_bias": round((float(img.mean()) - omean) / omean, 5), "seconds_to_rmse": levels,
               "curve": curve[:: max(1, len(curve) // 12)] + curve[-1:]}
        if kind == "cached":
            out.update(cache_record_bias=round(m.cache_bias, 4), train_loss=round(m.cache_train_loss, 4),
                       warmup_frames=args.ttr_warmup, unbiased_share=0.03, lr=1e-3,
                       train_records_per_frame=m.cache_train_samples)
        return out

    mk = run("megakernel")
    wf = run("wavefront")
    cached = run("cached")

    def ratio(a, b):
        return round(a / b, 2) if a and b else None

    return {"target_rmse": args.ttr_target, "unit": "s", "higher_is_better": False,
            "rmse": "sqrt(mean over crop-interior pixels x RGB of (I - I_oracle)^2), resolved linear film",
            "crop": [x0, y0, x1, y1], "oracle": {"renderer": "FP64 megakernel", "spp": npass * spp_pass,
                                                 "seconds": round(oracle_ms / 1000, 2),
                                                 "rmse_estimate": oracle_err, "mean": omean},
            "plain_megakernel": mk, "plain_wavefront": wf, "cached_wavefront": cached,
            "speedup": ratio(mk["seconds_to_target"], cached["seconds_to_target"]),
            "speedup_vs_plain_wavefront": ratio(wf["seconds_to_target"], cached["seconds_to_target"]),
            "speedup_by_rmse": {k: ratio(mk["seconds_to_rmse"][k], v) for k, v in cached["seconds_to_rmse"].items()},
            "speedup_vs_plain_wavefront_by_rmse": {k: ratio(wf["seconds_to_rmse"][k], v)
                                                   for k, v in cached["seconds_to_rmse"].items()},
            "wall_s": round(time.time() - t_start, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="stress", choices=sorted(WORKLOADS),
                    help="stress: glass + rough conductors, 1920x1080, 256 spp, 16 bounces (default); "
                         "displaced: displaced icosphere, 1024x1024, 64 spp, 8 bounces; small: its "
                         "256x256x16 spp level-6 version (quick check)")
    ap.add_argument("--small", action="store_true", help="same as --workload small")
    ap.add_argument("--skip-lbvh", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-ttr", action="store_true", help="leave out the time-to-RMSE block")
    ap.add_argument("--skip-displaced", action="store_true", help="leave out the displaced-icosphere figures")
    ap.add_argument("--skip-watertight", action="store_true", help="leave out the watertight-test render")
    ap.add_argument("--skip-instanced", action="store_true", help="leave out the instanced stress-scene figures")
    ap.add_argument("--skip-bdpt", action="store_true", help="leave out the bidirectional path tracing figures")
    ap.add_argument("--libm-double", type=int, default=None, choices=[0, 1],
                    help="set the renderer's libm_double option (float cos/sin/acos/log2 evaluated in double)")
    ap.add_argument("--integrator", type=int, default=1, choices=[0, 1], help="0 megakernel, 1 wavefront")
    ap.add_argument("--bvh-width", type=int, default=8, choices=[2, 8],
                    help="traversal structure: 8-wide compressed BVH or the binary LBVH")
    ap.add_argument("--lbvh-only", type=int, default=0, metavar="N",
                    help="only time the LBVH build over N random triangles (seed 1), both modes")
    ap.add_argument("--render-bvh", type=int, default=1, choices=[0, 1, 2],
                    help="tree the 8-wide BVH is collapsed from: 1 PLOC clustering with the SAH-optimal "
                         "collapse, 2 PLOC with the greedy collapse, 0 the LBVH itself")
    ap.add_argument("--pool", type=int, default=0, metavar="PATHS",
                    help="wavefront path-state pool capacity (0: the renderer's automatic size)")
    ap.add_argument("--views64", action="store_true", help="64 batched uneven views (autotuned, with the cache)")
    ap.add_argument("--views-oracle-spp", type=int, default=1024,
                    help="spp of the FP64 oracle crops the 64 views' RMSE is taken against")
    ap.add_argument("--bdpt-only", action="store_true",
                    help="only the bidirectional path tracing figures (the bdpt key)")
    ap.add_argument("--mlp-only", action="store_true",
                    help="radiance-cache network alone: inference over 1920x1080 queries, one 65,536-sample training step")
    ap.add_argument("--time-to-rmse", action="store_true",
                    help="only the time-to-RMSE block (megakernel, wavefront, cached wavefront)")
    ap.add_argument("--ttr-target", type=float, default=1e-2)
    ap.add_argument("--ttr-crop", type=int, nargs=2, default=[192, 108])
    ap.add_argument("--ttr-oracle-spp", type=int, default=65536)
    ap.add_argument("--ttr-spp-plain", type=int, default=8, help="spp per frame of the plain megakernel")
    ap.add_argument("--ttr-spp-wavefront", type=int, default=8, help="spp per frame of the plain wavefront")
    ap.add_argument("--ttr-spp-cached", type=int, default=4, help="spp per frame of the cached wavefront")
    ap.add_argument("--ttr-warmup", type=int, default=8)
    ap.add_argument("--ttr-max-seconds", type=float, default=60.0)
    args = ap.parse_args()
    wl = WORKLOADS["small" if args.small else args.workload]
    if args.time_to_rmse:
        import lighttransportsimulation_gb300 as lts
        ctx = lts.Context(0)
        print(json.dumps({"time_to_rmse": time_to_rmse(args, ctx)}))
        ctx.close()
        return
    if args.views64:
        views64(args)
        return
    if args.lbvh_only:
        import lighttransportsimulation_gb300 as lts
        ctx = lts.Context(0)
        print(json.dumps(lbvh_bench(ctx, args.lbvh_only, args.steps, args.warmup, (lts.BVH_REFERENCE, lts.BVH_SORTED),
                                    measured_peaks()[0])))
        ctx.close()
        return
    if args.mlp_only:
        import lighttransportsimulation_gb300 as lts
        ctx = lts.Context(0)
        print(json.dumps({"mlp": mlp_bench(ctx, args.steps, args.warmup, measured_peaks()[0])}))
        ctx.close()
        return
    if args.bdpt_only:
        import lighttransportsimulation_gb300 as lts
        ctx = lts.Context(0)
        print(json.dumps({"bdpt": bdpt_extra(args, ctx)}))
        ctx.close()
        return
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_gpu(args, wl)


if __name__ == "__main__":
    main()
