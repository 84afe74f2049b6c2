"""Failure paths on the GPU, made without faulting it: an allocation cap (LTS_MAX_DEVICE_MB) that
makes a scene upload fail part way, and bounded waits that are made to run out by lowering their
poll limit.  Each case runs in a child process, so that the cap and the lowered limit stay out
of the other tests."""
import json
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu
ERR_OOM, ERR_STATE, ERR_DEVICE = 5, 7, 8  # LTS_ERR_* of include/lts_capi.h

_OOM_CHILD = r"""
import ctypes, json, sys, tempfile
sys.path.insert(0, sys.argv[1])
import numpy as np
import lighttransportsimulation_gb300 as lts
from lighttransportsimulation_gb300 import scenes
out = {}
big = tempfile.mkdtemp()
scenes.write_displaced(big, level=7)          # 327,692 triangles: tables far above the cap
small = tempfile.mkdtemp()
sc, sub = scenes.write_box_sphere(small)      # 5,132 triangles: fits
ctx = lts.Context(0)
try:
    lts.Scene.parse(ctx, big, "box", "displaced", 64, 64)
    out["big"] = 0
except lts.LtsError as e:
    out["big"] = e.code
info = lts.SceneInfo()
out["info_after_fail"] = ctx.lib.lts_scene_info_get(ctx.h, ctypes.byref(info))
desc = lts.RenderDesc(spp=1, max_bounce=2, rr_start=1, seed=0, integrator=1, x0=0, y0=0, x1=8, y1=8,
                      record_samples=0, bvh_mode=lts.BVH_SORTED)
out["render_after_fail"] = ctx.lib.lts_render(ctx.h, ctypes.byref(desc), None)
fx = np.load(sys.argv[2])
w, h, spp, maxb, rr, seed, x0, y0, x1, y1 = (int(v) for v in fx["meta"])
s = lts.Scene.parse(ctx, small, sc, sub, w, h)
r = lts.PathTracingIntegrator(maxb, rr, s, integrator=lts.INTEGRATOR_MEGAKERNEL).render(
    spp, seed, crop=(x0, y0, x1, y1), record=True, film=False)
L, Lr = r["L"].reshape(-1, 3), fx["L"].reshape(-1, 3)
same = r["sig"].reshape(-1) == fx["sig"].reshape(-1)
ok = np.all(np.abs(L - Lr) <= 1e-4 * np.abs(Lr) + 1e-6, axis=1)
out["divergent"] = float(1 - same.mean())
out["outside"] = float(1 - ok[same].mean())
out["device_mb"] = ctx.metrics().device_bytes / 2**20
ctx.close()
print("RESULT " + json.dumps(out))
"""

_WAIT_CHILD = r"""
import json, sys, tempfile
sys.path.insert(0, sys.argv[1])
import numpy as np
import lighttransportsimulation_gb300 as lts
from lighttransportsimulation_gb300 import scenes
out = {}
ctx = lts.Context(0)
ctx.set_option("debug_spin_limit", 1000)
for which in (0, 1):
    rc = ctx.lib.lts_debug_wait_timeout(ctx.h, which)
    out[f"rc{which}"] = rc
    out[f"msg{which}"] = ctx.lib.lts_last_error(ctx.h).decode()
ctx.set_option("debug_spin_limit", 0)
# the context is still usable: a bit-exact LBVH build of the box scene after the timeouts
d = tempfile.mkdtemp()
sc, sub = scenes.write_box_sphere(d)
fx = np.load(sys.argv[2])
meta = np.load(sys.argv[3])["meta"]
s = lts.Scene.parse(ctx, d, sc, sub, int(meta[0]), int(meta[1]))
b = s.create_bvh_tree(lts.BVH_REFERENCE)
out["lbvh_equal"] = all(bool(np.array_equal(b[k], fx[k])) for k in
                        ("sorted_codes", "sorted_ids", "node_key", "node_left", "node_right"))
out["bounds_equal"] = bool(np.array_equal(b["node_bounds"].view(np.uint32), fx["node_bounds"].view(np.uint32)))
ctx.close()
print("RESULT " + json.dumps(out))
"""


def _child(code, *args, env=None):
    p = subprocess.run([sys.executable, "-c", code, ROOT, *args], capture_output=True, text=True, timeout=600,
                       env={**os.environ, **(env or {})})
    assert p.returncode == 0, p.stderr[-3000:]
    line = [x for x in p.stdout.splitlines() if x.startswith("RESULT ")][-1]
    return json.loads(line[len("RESULT "):])


def test_upload_over_the_cap_fails_cleanly(built_lib):
    """A scene whose tables exceed LTS_MAX_DEVICE_MB fails with LTS_ERR_OOM part way through its
    upload; the context then holds no scene (queries and renders return LTS_ERR_STATE instead of
    reading half-written or freed tables), and the next load renders the reference's samples."""
    r = _child(_OOM_CHILD, os.path.join(GOLDEN, "render_box_sphere.npz"), env={"LTS_MAX_DEVICE_MB": "24"})
    assert r["big"] == ERR_OOM
    assert r["info_after_fail"] == ERR_STATE
    assert r["render_after_fail"] == ERR_STATE
    assert r["divergent"] <= 0.01 and r["outside"] <= 0.005, r
    assert r["device_mb"] <= 24


def test_bounded_waits_run_out_and_the_context_survives(built_lib):
    """With the poll limit lowered, a look-back-style wait on a flag nothing sets and an
    mbarrier wait on a phase nothing completes both give up: the kernels set their error flags
    (DEV_ERR_LOOKBACK_TIMEOUT = 0x1, DEV_ERR_MMA_TIMEOUT = 0x20) and return, the calls return
    LTS_ERR_DEVICE, and the same context then builds the reference's LBVH bit for bit."""
    r = _child(_WAIT_CHILD, os.path.join(GOLDEN, "lbvh_box_sphere.npz"), os.path.join(GOLDEN, "render_box_sphere.npz"))
    assert r["rc0"] == ERR_DEVICE and r["msg0"].endswith("0x1"), r
    assert r["rc1"] == ERR_DEVICE and r["msg1"].endswith("0x20"), r
    assert r["lbvh_equal"] and r["bounds_equal"]
