"""CPU tests of the C-ABI library: it loads, exports every symbol the header declares, and its
host-side loader reproduces the reference's parseScene outputs bit for bit."""
import os
import re
import struct

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def test_library_exports_header_symbols(built_lib):
    import ctypes
    import lighttransportsimulation_gb300 as lts
    hdr = open(os.path.join(ROOT, "include", "lts_capi.h")).read()
    declared = sorted(set(re.findall(r"\b(lts_[a-z0-9_]+)\s*\(", hdr)))
    lib = ctypes.CDLL(built_lib)
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(lts.EXPORTS) == declared


@pytest.mark.parametrize("kind", ["box_sphere", "materials", "closeup_diamond", "closeup_moai", "bigbox_diamond"])
def test_loader_matches_reference(built_lib, scene_dirs, kind):
    """The host loader against the reference's parseScene: world triangles (bit patterns, or
    their sha256 for large meshes), camera and light distribution, on the synthetic parity
    scenes and the reference's own shipped scenes."""
    import hashlib

    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs[kind]
    fx = np.load(os.path.join(GOLDEN, f"lbvh_{kind}.npz"))
    meta = np.load(os.path.join(GOLDEN, f"render_{kind}.npz"))["meta"]
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d, sc, sub, int(meta[0]), int(meta[1]))
    tri = s.triangles().reshape(-1)
    if "tri_p" in fx.files:
        assert np.array_equal(tri.view(np.uint32), fx["tri_p"].view(np.uint32))
    else:
        assert hashlib.sha256(tri.tobytes()).hexdigest() == str(fx["tri_p_sha256"])
    assert np.array_equal(s.camera().view(np.uint32), fx["camera"].view(np.uint32))
    func, cdf = s.light_distribution()
    assert np.array_equal(func.view(np.uint32), fx["light_func"].view(np.uint32))
    assert np.array_equal(cdf.view(np.uint32), fx["light_cdf"].view(np.uint32))
    assert s.light_count == len(fx["light_flags"])


def test_app_params(tmp_path, built_lib):
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    p = tmp_path / "app.params"
    scenes.write_app_params(p, 320, 200, 16, 5, 3, 1, "out", "res/a", "res/b")
    d = lts.read_application_parameters(str(p))
    assert (d["width"], d["height"], d["spp"], d["max_bounce"], d["rr_start"], d["format"]) == (320, 200, 16, 5, 3, 1)
    assert d["output"] == "out.pfm" and d["scene"] == "res/a" and d["subject"] == "res/b"
    with pytest.raises(lts.LtsError):
        lts.read_application_parameters(str(tmp_path / "missing.params"))


def _load_err(d, sc, sub):
    import lighttransportsimulation_gb300 as lts
    ctx = lts.Context(-1)
    with pytest.raises(lts.LtsError) as e:
        lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    return e.value.code


def test_loader_errors(tmp_path, built_lib):
    from lighttransportsimulation_gb300 import scenes
    d = str(tmp_path)
    sc, sub = scenes.write_box_sphere(d)
    assert _load_err(d, "nope", sub) == 2                        # missing .scene -> IO
    b = os.path.join(d, "sphere.bin")
    raw = open(b, "rb").read()
    open(b, "wb").write(raw[:100])
    assert _load_err(d, sc, sub) == 3                            # truncated .bin -> PARSE
    bad = bytearray(raw)
    ntri, npnt, nuv, nn = struct.unpack("<4i", raw[:16])
    off = 16 + 12 * npnt + 8 * nuv + 12 * nn
    bad[off:off + 4] = struct.pack("<i", npnt + 5)
    open(b, "wb").write(bytes(bad))
    assert _load_err(d, sc, sub) == 3                            # vertex index out of range
    open(b, "wb").write(raw)
    txt = open(os.path.join(d, "sphere.subject")).read()
    open(os.path.join(d, "sphere.subject"), "w").write(txt.replace("L\tc\t0.8 0.8 0.8", "L\ti\t0"))
    assert _load_err(d, sc, sub) == 3                            # image texture without an image
    img = txt.replace("L\tc\t0.8 0.8 0.8", "L\ti\t0").replace("0\n", "1\t0\ttex.jpg\n", 1)
    open(os.path.join(d, "sphere.subject"), "w").write(img)
    assert _load_err(d, sc, sub) == 2                            # missing image file -> IO
    open(os.path.join(d, "tex.jpg"), "wb").write(b"\xff\xd8\xff\xe0" + bytes(60))
    assert _load_err(d, sc, sub) == 3                            # malformed JPEG -> PARSE
    open(os.path.join(d, "tex.jpg"), "wb").write(b"GIF89a" + bytes(60))
    assert _load_err(d, sc, sub) == 6                            # neither PNG nor JPEG -> UNSUPPORTED
    open(os.path.join(d, "sphere.subject"), "w").write("0\n1\tsphere\n")
    assert _load_err(d, sc, sub) == 3                            # premature end of file


def test_host_only_context_has_no_device_path(built_lib, scene_dirs):
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["box_sphere"]
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d, sc, sub, 32, 32)
    with pytest.raises(lts.LtsError) as e:
        s.create_bvh_tree(lts.BVH_REFERENCE)
    assert e.value.code == 7


def test_reloads_and_a_failed_load_keep_the_scene(built_lib, scene_dirs, tmp_path):
    """A load that fails leaves the loaded scene as it was; loads of scenes of other sizes in
    turn (the context parses each into the previous scene's tables) give the same triangles as
    a fresh context."""
    import lighttransportsimulation_gb300 as lts
    d1, sc1, sub1 = scene_dirs["box_sphere"]
    d2, sc2, sub2 = scene_dirs["materials"]
    ref = {}
    for key, (d, sc, sub) in (("a", (d1, sc1, sub1)), ("b", (d2, sc2, sub2))):
        c = lts.Context(-1)
        ref[key] = lts.Scene.parse(c, d, sc, sub, 32, 32).triangles().copy()
        c.close()
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d1, sc1, sub1, 32, 32)
    with pytest.raises(lts.LtsError):
        lts.Scene.parse(ctx, str(tmp_path), "nope", None, 32, 32)
    assert np.array_equal(s.triangles().view(np.uint32), ref["a"].view(np.uint32))
    for key, (d, sc, sub) in (("b", (d2, sc2, sub2)), ("a", (d1, sc1, sub1)), ("b", (d2, sc2, sub2))):
        s = lts.Scene.parse(ctx, d, sc, sub, 32, 32)
        assert np.array_equal(s.triangles().view(np.uint32), ref[key].view(np.uint32))
    ctx.close()


def _scene_state(s):
    func, cdf = s.light_distribution()
    return {"info": s.query_info(), "tri": s.triangles().view(np.uint32).copy(),
            "cam": s.camera().view(np.uint32).copy(), "func": func.view(np.uint32).copy(),
            "cdf": cdf.view(np.uint32).copy()}


def test_failed_load_part_way_keeps_the_scene(built_lib, scene_dirs, tmp_path):
    """Loads that fail after the scene header -- a truncated mesh, a vertex index out of range,
    an unknown material code -- have already written into the spare tables (materials cleared,
    tables resized); the loaded scene's info, triangles, camera and light distribution still
    equal a fresh context's."""
    import shutil

    import lighttransportsimulation_gb300 as lts
    d1, sc1, sub1 = scene_dirs["materials"]
    fresh = lts.Context(-1)
    want = _scene_state(lts.Scene.parse(fresh, d1, sc1, sub1, 40, 24))
    fresh.close()

    d2 = str(tmp_path / "broken")
    shutil.copytree(scene_dirs["box_sphere"][0], d2)
    sc2, sub2 = scene_dirs["box_sphere"][1], scene_dirs["box_sphere"][2]
    b = os.path.join(d2, "sphere.bin")
    raw = open(b, "rb").read()
    ntri, npnt, nuv, nn = struct.unpack("<4i", raw[:16])
    off = 16 + 12 * npnt + 8 * nuv + 12 * nn
    bad_index = bytearray(raw)
    bad_index[off + 36 * (ntri - 1):off + 36 * (ntri - 1) + 4] = struct.pack("<i", npnt + 7)
    subj = os.path.join(d2, "sphere.subject")
    txt = open(subj).read()
    breakers = [
        lambda: open(b, "wb").write(raw[:off + 36 * (ntri // 2)]),     # mesh ends mid index table
        lambda: open(b, "wb").write(bytes(bad_index)),                  # last triangle out of range
        lambda: (open(b, "wb").write(raw),
                 open(subj, "w").write(txt.replace("L\tc\t0.8 0.8 0.8", "Q\tc\t0.8 0.8 0.8"))),  # unknown material
    ]
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d1, sc1, sub1, 40, 24)
    for brk in breakers:
        brk()
        with pytest.raises(lts.LtsError) as e:
            lts.Scene.parse(ctx, d2, sc2, sub2, 64, 64)
        assert e.value.code == 3
        got = _scene_state(s)
        assert got["info"] == want["info"]
        for k in ("tri", "cam", "func", "cdf"):
            assert np.array_equal(got[k], want[k]), k
    ctx.close()


def test_point_light_grammar_extension(built_lib, tmp_path):
    """`pointLights N  px py pz Ir Ig Ib ...` after the infinite-light record (no counterpart in
    the reference): the lights table holds the ceiling triangles, then the point lights, then
    the infinite light; a point light's power is 4 pi I (Light.cuh:83-85), so its entry of the
    light distribution is the luminance of 4 pi I.  Where the reference build exists, it loads
    the same file without the point lights, and every other entry matches it bit for bit."""
    import subprocess

    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from oracle import ltsd
    d = str(tmp_path)
    sc, sub = scenes.write_point_lights(d)
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    func, cdf = s.light_distribution()
    assert s.info["lights"] == 2 + len(scenes.POINT_LIGHTS) + 1 and s.info["has_infinite"] == 1
    for k, (_, inten) in enumerate(scenes.POINT_LIGHTS):
        v = np.float32(4 * np.pi)
        pw = [np.float32(c) * v for c in inten]
        want = np.float32(0.212671) * pw[0] + np.float32(0.715160) * pw[1] + np.float32(0.072169) * pw[2]
        assert func[2 + k] == pytest.approx(float(want), rel=1e-6)
    # a file whose trailing text is not the keyword keeps the reference's reading
    txt = open(os.path.join(d, sc + ".scene")).read()
    open(os.path.join(d, "plain.scene"), "w").write(txt[: txt.index("pointLights")] + "// trailing note\n")
    s2 = lts.Scene.parse(ctx, d, "plain", sub, 64, 64)
    assert s2.info["lights"] == 3
    ref = os.path.join(ROOT, "oracle", "_ref", "lts_ref")
    if os.path.exists(ref):
        out = str(tmp_path / "b.ltsd")
        subprocess.run([ref, "bvh", d + "/", sc, sub, out, "64", "64"], check=True)
        r = ltsd.read(out)
        keep = np.r_[0:2, 2 + len(scenes.POINT_LIGHTS):len(func)]
        np.testing.assert_array_equal(r["light_func"], func[keep])
        np.testing.assert_array_equal(r["light_func"], s2.light_distribution()[0])
    ctx.close()


def _app_setup(tmp_path):
    from lighttransportsimulation_gb300 import build, scenes
    d = str(tmp_path)
    sc, sub = scenes.write_box_sphere(d)
    scenes.write_app_params(os.path.join(d, "app.params"), 64, 48, 4, 5, 3, 1, "out", sc, sub)
    return d, build.APP


def test_host_program_runs_on_a_host_only_context(built_lib, tmp_path):
    """The thin C host program (host/render_app.c, the reference's main over the C-ABI) compiles,
    links, reads app.params and parses the scene; with --device -1 its render step reports that it
    needs a GPU (LTS_ERR_STATE) instead of exiting inside the library."""
    import subprocess
    d, app = _app_setup(tmp_path)
    assert os.path.exists(app)
    r = subprocess.run([app, d, "--device", "-1"], capture_output=True, text=True)
    assert r.returncode == 7, r.stderr
    assert "5132 triangles" in r.stdout and "64x48, 4 spp, 5 bounces" in r.stdout
    assert "status 7" in r.stderr
    r = subprocess.run([app, str(tmp_path / "missing")], capture_output=True, text=True)
    assert r.returncode == 2   # LTS_ERR_IO: no app.params


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_loader_matches_reference_on_the_bench_scene(built_lib, tmp_path):
    """The displaced-icosphere bench scene (1,310,732 triangles): the loader's world triangles,
    camera and light distribution have the sha256 digests of the reference's parseScene outputs
    (tests/golden/digest_displaced.npz, made by oracle/_ref/lts_ref)."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from conftest import scene_digest
    z = np.load(os.path.join(GOLDEN, "digest_displaced.npz"))
    d = str(tmp_path)
    scenes.write_displaced(d, level=8)
    assert sorted(z["scene_digest"]) == sorted(scene_digest(d)), "scene generator drifted"
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d, "box", "displaced", 1024, 1024)
    assert s.info["triangles"] == int(z["n"])
    assert _sha(s.triangles().reshape(-1)) == str(z["tri_p"])
    assert _sha(s.camera()) == str(z["camera"])
    func, cdf = s.light_distribution()
    assert _sha(func) == str(z["light_func"]) and _sha(cdf) == str(z["light_cdf"])
    ctx.close()


def test_loader_matches_reference_on_the_dragon_scene(built_lib, tmp_path):
    """The reference's JPEG-textured subject res/blackDragon on res/platforms/closeupPlane (37,986
    triangles, 480 x 270): world triangles, camera and light distribution have the sha256 digests
    of the reference's parseScene outputs (tests/golden/digest_dragon.npz; taken with the
    subject's texture replaced by a constant, since the reference's loader crashes in its texture
    set-up on this subject), and the texture's level 0 is the reference reader's decoding of
    res/blackDragon.jpg (its digest in tests/golden/jpeg_golden.npz)."""
    import lighttransportsimulation_gb300 as lts
    from conftest import write_dragon
    z = np.load(os.path.join(GOLDEN, "digest_dragon.npz"))
    g = np.load(os.path.join(GOLDEN, "jpeg_golden.npz"))
    root, sc, sub = write_dragon(str(tmp_path))
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, root, sc, sub, 480, 270)
    assert s.info["triangles"] == int(z["n"]) and s.info["images"] == 1
    assert _sha(s.triangles().reshape(-1)) == str(z["tri_p"])
    assert _sha(s.camera()) == str(z["camera"])
    func, cdf = s.light_distribution()
    assert _sha(func) == str(z["light_func"]) and _sha(cdf) == str(z["light_cdf"])
    tex, levels = s.image(0, 0)
    assert levels == 9 and _sha(tex.reshape(512, 512, 3)) == str(g["dragon_sha256"])
    ctx.close()


def test_instances_grammar_extension(built_lib, tmp_path):
    """`instances K` and per instance `meshIndex tx ty tz s` after the infinite-light record (no
    counterpart in the reference): mesh entry meshIndex holds its file's triangles at p * s + t,
    rounded in float32 as written; entries naming the same file share one prototype.  The scene's
    triangle table is the flattened one (what the oracle and the flat BVH see), equal to the plain
    stress scene's up to the rounding of where the placement happens.  Malformed records fail
    with LTS_ERR_PARSE."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    d = str(tmp_path)
    sc, sub = scenes.write_stress_scene(d, rings=16, segs=32)
    si, ss = scenes.write_stress_scene(d, rings=16, segs=32, instanced=True)
    ctx = lts.Context(-1)
    plain = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    tp, ip = plain.triangles(), plain.info
    inst = lts.Scene.parse(ctx, d, si, ss, 64, 64)
    ti, ii = inst.triangles(), inst.info
    assert ii["instances"] == 8 and ii["prototypes"] == 1 and ip["instances"] == 0
    assert ii["triangles"] == ip["triangles"] and ii["lights"] == ip["lights"]
    np.testing.assert_allclose(ti, tp, atol=2e-7, rtol=0)
    # every instanced triangle is the file's, scaled then moved, in float32
    v, f = scenes.uv_sphere(16, 32)
    v32 = v.astype(np.float32)
    per = len(f)
    glass = per  # mesh entry 0 (the glass sphere) comes first
    lines = open(os.path.join(d, si + ".scene")).read().split("instances")[1].split("\n")[1:9]
    for k, line in enumerate(lines):
        m, t, s = line.split("\t")
        t = np.array([np.float32(x) for x in t.split()], np.float32)
        want = v32[f] * np.float32(s) + t
        got = ti[glass + k * per: glass + (k + 1) * per]
        assert int(m) == 1 + k and np.array_equal(got, want)
    txt = open(os.path.join(d, si + ".scene")).read()
    head, tail = txt.split("instances")
    for bad in ("instances\t1\n14\t0 0 0\t1\n",     # mesh index out of range (14 entries)
                "instances\t1\n13\t0 0 0\t1\n",     # the area light's mesh (emissive)
                "instances\t2\n1\t0 0 0\t1\n1\t0 0 0\t1\n",  # the same entry twice
                "instances\t1\n1\t0 0 0\t0\n",      # scale not > 0
                "instances\t1\n1\t0 0\n"):          # premature end
        open(os.path.join(d, "bad.scene"), "w").write(head + bad)
        assert _load_err(d, "bad", ss) == 3, bad
    # a subject mesh is instanced only under the identity subject transform
    lines = txt.split("\n")
    lines[1] = "0 0 0\t0 1 0\t0.5\t1"
    open(os.path.join(d, "rot.scene"), "w").write("\n".join(lines))
    assert _load_err(d, "rot", ss) == 3
    ctx.close()
