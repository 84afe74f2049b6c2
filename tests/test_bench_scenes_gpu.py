"""Per-sample parity on the benchmarked scenes themselves, against the oracle's CPU port run on
this host (the port is bit-exact to the reference on every scene the reference loads; the
stress scene's conductors are a grammar extension the reference cannot load):

  * the displaced-icosphere render of the bench (1,310,732 triangles, wrinkled texture, 1024 x 1024,
    8 bounces, roulette from 3): a 32 x 32 crop at 4 spp;
  * the material-stress scene at full size (2,350,092 triangles: displaced glass, eight rough
    conductors, marble floor, area + infinite light; 1920 x 1080, 16 bounces, roulette from 4): a
    32 x 32 crop at 4 spp.

Same rule as tests/test_render_gpu.py: samples whose event hash (renderer's or FP64 renderer's)
differs from the port's are divergent (at most 1 %); every other sample within 1e-4 relative plus
1e-6 plus four times the port's own distance from the FP64 value of the same path."""
import os
import subprocess

import numpy as np
import pytest

from test_render_gpu import check_samples

pytestmark = pytest.mark.gpu

CASES = {
    "displaced_1024": dict(w=1024, h=1024, spp=4, maxb=8, rr=3, seed=0, crop=(496, 560, 528, 592)),
    "stress_1080p": dict(w=1920, h=1080, spp=4, maxb=16, rr=4, seed=0, crop=(944, 524, 976, 556)),
}


@pytest.fixture(scope="module")
def bench_scenes(tmp_path_factory):
    from lighttransportsimulation_gb300 import scenes
    out = {}
    d = str(tmp_path_factory.mktemp("displaced"))
    scenes.write_displaced(d, level=8)
    out["displaced_1024"] = (d, "box", "displaced")
    d = str(tmp_path_factory.mktemp("stress"))
    scenes.write_stress_scene(d)
    out["stress_1080p"] = (d, "stress", "stress")
    return out


@pytest.mark.parametrize("case", list(CASES))
def test_bench_scene_crop_matches_the_port(built_lib, port_exe, bench_scenes, tmp_path, case):
    import lighttransportsimulation_gb300 as lts
    from oracle import ltsd
    c = CASES[case]
    d, sc, sub = bench_scenes[case]
    x0, y0, x1, y1 = c["crop"]
    out = str(tmp_path / "port.ltsd")
    args = (port_exe, "render", d + "/", sc, sub, out, c["w"], c["h"], c["spp"], c["maxb"], c["rr"], c["seed"],
            x0, y0, x1, y1, os.cpu_count(), 0, 0)
    subprocess.run([str(a) for a in args], check=True)
    ref = ltsd.read(out)
    Lr, sr = ref["L"].reshape(-1, 3), ref["sig"].reshape(-1)
    ctx = lts.Context(0)
    try:
        s = lts.Scene.parse(ctx, d, sc, sub, c["w"], c["h"])
        res = {}
        for integ in (lts.INTEGRATOR_FP64, lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
            r = lts.PathTracingIntegrator(c["maxb"], c["rr"], s, integrator=integ).render(
                c["spp"], c["seed"], crop=(x0, y0, x1, y1), record=True, film=False)
            res[integ] = (r["L"].reshape(-1, 3).copy(), r["sig"].reshape(-1).copy())
    finally:
        ctx.close()
    L64, s64 = res[lts.INTEGRATOR_FP64]
    assert Lr.mean() > 0
    for integ in (lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
        L, sig = res[integ]
        check_samples(L, sig, Lr, sr, L64, s64, f"{case} integrator={integ}")
