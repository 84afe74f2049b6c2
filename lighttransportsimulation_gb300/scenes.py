"""Seeded synthetic scenes written in the reference's own input formats.

Every scene is a `.scene` file, an optional `.subject` file and `.bin` meshes, laid out by
the grammar of core/SceneLoader.cuh:195-253 and core/FileIO.cuh:170-206 of the reference
(tierChampion/LightTransportSimulation), so the same files drive the reference build, the
CPU oracle and this renderer.  No public benchmark data is involved.

Workloads (sizes are the ones the benchmarks are quoted on):
  box_sphere   256x256, 16 spp, 5 bounces, roulette from 3: an open-front box [-1,1]^3 of
               5 Lambertian walls (10 tris; white 0.7, left (0.7,0.1,0.1), right
               (0.1,0.7,0.1)), a 0.5x0.5 ceiling light quad (2 tris, Le 10) and a level-4
               icosphere (5120 tris, r 0.5, albedo 0.8): 5132 triangles.
  displaced    the same box holding a level-8 icosphere (1,310,720 tris) radially displaced
               by 0.1 * fbm(8 octaves, omega 0.5) with a wrinkled Lambertian texture
               (8 octaves, omega 0.5); 1024x1024, 64 spp, 8 bounces.
  random_tris  N triangles with centroids U[0,1)^3 and vertices centroid + N(0, 1e-3)^3, FP32,
               seed 1 (the LBVH build benchmark, 1M and 16M).
  stress       material and divergence stress: in the same box, a glass (IOR 1.5) lat-long sphere
               of 512 x 256 segments (261,120 tris) displaced by 0.1 * fbm(8, 0.5); eight rough
               conductor spheres of the same tessellation (Trowbridge-Reitz, alpha U[0.05, 0.5]
               per copy, positions seeded with 2) written as eight pre-transformed meshes; a
               marble Lambertian floor (8 octaves, omega 0.5, scale 4); the ceiling area light and
               a constant infinite light of 0.5.  1920x1080, 256 spp, 16 bounces, roulette from 4.
"""
import os

import numpy as np

# ----------------------------------------------------------------------------- .bin meshes


def write_bin(path, p, n, idx_p, idx_n, uv=None, idx_uv=None):
    """Write a mesh in the reference's .bin layout (FileIO.cuh:20-45):
    int32 nTri, nP, nUV, nN; float3 P[nP]; float2 UV[nUV]; float3 N[nN]; int32 idx[9 nTri]
    with per-corner (p, uv, n) indices.  -0.0 coordinates are written as +0.0."""
    p = np.ascontiguousarray(p, dtype=np.float32) + np.float32(0.0)
    n = np.ascontiguousarray(n, dtype=np.float32) + np.float32(0.0)
    ntri = idx_p.shape[0]
    if uv is None:
        uv = np.zeros((0, 2), np.float32)
        idx_uv = np.zeros_like(idx_p)
    idx = np.empty((ntri, 3, 3), np.int32)
    idx[:, :, 0] = idx_p
    idx[:, :, 1] = idx_uv
    idx[:, :, 2] = idx_n
    with open(path, "wb") as f:
        f.write(np.array([ntri, p.shape[0], uv.shape[0], n.shape[0]], np.int32).tobytes())
        f.write(p.tobytes())
        f.write(np.ascontiguousarray(uv, np.float32).tobytes())
        f.write(n.tobytes())
        f.write(idx.tobytes())


def read_bin(path):
    with open(path, "rb") as f:
        hdr = np.frombuffer(f.read(16), np.int32)
        ntri, np_, nuv, nn = (int(x) for x in hdr)
        p = np.frombuffer(f.read(12 * np_), np.float32).reshape(np_, 3)
        uv = np.frombuffer(f.read(8 * nuv), np.float32).reshape(nuv, 2)
        n = np.frombuffer(f.read(12 * nn), np.float32).reshape(nn, 3)
        idx = np.frombuffer(f.read(36 * ntri), np.int32).reshape(ntri, 3, 3)
    return p, uv, n, idx


def quad(c, du, dv):
    """Two triangles spanning corner c, c+du, c+du+dv, c+dv (counter-clockwise about du x dv)."""
    c, du, dv = (np.asarray(x, np.float64) for x in (c, du, dv))
    p = np.stack([c, c + du, c + du + dv, c + dv])
    tris = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    nrm = np.cross(du, dv)
    nrm /= np.linalg.norm(nrm)
    return p, tris, nrm


def write_quads(path, quads):
    ps, ns, ip, inn = [], [], [], []
    off = 0
    for k, (c, du, dv) in enumerate(quads):
        p, t, nrm = quad(c, du, dv)
        ps.append(p)
        ns.append(nrm[None, :])
        ip.append(t + off)
        inn.append(np.full_like(t, k))
        off += 4
    write_bin(path, np.concatenate(ps), np.concatenate(ns), np.concatenate(ip), np.concatenate(inn))


def icosphere(level):
    """Vertices (unit sphere, float64) and triangles of a subdivided icosahedron; the four
    children of each face are emitted contiguously, so triangle order is spatially coherent."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (nv + 1) + e[:, 1]
        ukey, inv = np.unique(key, return_inverse=True)
        a, b = ukey // (nv + 1), ukey % (nv + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + nv  # midpoints of (v0v1, v1v2, v2v0)
        v = np.concatenate([v, mid])
        a0, a1, a2 = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.stack([np.stack([a0, m01, m20], 1), np.stack([a1, m12, m01], 1),
                      np.stack([a2, m20, m12], 1), np.stack([m01, m12, m20], 1)], 1).reshape(-1, 3)
    return v, f.astype(np.int32)


# ----------------------------------------------------------------------------- noise (fbm)

_PERM = None


def _perm():
    """The fixed 512-entry improved-Perlin permutation of textures/Procedural.cuh:79-107,
    reconstructed from Ken Perlin's published 2002 reference permutation (the same table)."""
    global _PERM
    if _PERM is None:
        p = [151, 160, 137, 91, 90, 15, 131, 13, 201, 95, 96, 53, 194, 233, 7, 225, 140, 36, 103, 30, 69,
             142, 8, 99, 37, 240, 21, 10, 23, 190, 6, 148, 247, 120, 234, 75, 0, 26, 197, 62, 94, 252,
             219, 203, 117, 35, 11, 32, 57, 177, 33, 88, 237, 149, 56, 87, 174, 20, 125, 136, 171, 168,
             68, 175, 74, 165, 71, 134, 139, 48, 27, 166, 77, 146, 158, 231, 83, 111, 229, 122, 60, 211,
             133, 230, 220, 105, 92, 41, 55, 46, 245, 40, 244, 102, 143, 54, 65, 25, 63, 161, 1, 216, 80,
             73, 209, 76, 132, 187, 208, 89, 18, 169, 200, 196, 135, 130, 116, 188, 159, 86, 164, 100,
             109, 198, 173, 186, 3, 64, 52, 217, 226, 250, 124, 123, 5, 202, 38, 147, 118, 126, 255, 82,
             85, 212, 207, 206, 59, 227, 47, 16, 58, 17, 182, 189, 28, 42, 223, 183, 170, 213, 119, 248,
             152, 2, 44, 154, 163, 70, 221, 153, 101, 155, 167, 43, 172, 9, 129, 22, 39, 253, 19, 98,
             108, 110, 79, 113, 224, 232, 178, 185, 112, 104, 218, 246, 97, 228, 251, 34, 242, 193, 238,
             210, 144, 12, 191, 179, 162, 241, 81, 51, 145, 235, 249, 14, 239, 107, 49, 192, 214, 31, 181,
             199, 106, 157, 184, 84, 204, 176, 115, 121, 50, 45, 127, 4, 150, 254, 138, 236, 205, 93,
             222, 114, 67, 29, 24, 72, 243, 141, 128, 195, 78, 66, 215, 61, 156, 180]
        _PERM = np.array(p + p, np.int64)
    return _PERM


def perlin(pts):
    """Improved Perlin noise (Perlin 2002) at float32 points, vectorised: weights
    6t^5-15t^4+10t^3 and the 12+4 gradient directions of the published method."""
    perm = _perm()
    pts = np.asarray(pts, np.float32)
    fl = np.floor(pts)
    d = (pts - fl).astype(np.float32)
    i = fl.astype(np.int64) & 255

    def grad(ix, iy, iz, dx, dy, dz):
        h = perm[perm[perm[ix] + iy] + iz] & 15
        u = np.where((h < 8) | (h == 12) | (h == 13), dx, dy)
        v = np.where((h < 4) | (h == 12) | (h == 13), dy, dz)
        return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)

    dx, dy, dz = d[:, 0], d[:, 1], d[:, 2]
    ix, iy, iz = i[:, 0], i[:, 1], i[:, 2]
    one = np.float32(1)
    w = {}
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                w[a, b, c] = grad(ix + a, iy + b, iz + c, dx - a * one, dy - b * one, dz - c * one)

    def fade(t):
        t3 = t * t * t
        t4 = t3 * t
        return 6 * t4 * t - 15 * t4 + 10 * t3

    def lerp(t, a, b):
        return (1 - t) * a + t * b

    wx, wy, wz = fade(dx), fade(dy), fade(dz)
    x00 = lerp(wx, w[0, 0, 0], w[1, 0, 0])
    x10 = lerp(wx, w[0, 1, 0], w[1, 1, 0])
    x01 = lerp(wx, w[0, 0, 1], w[1, 0, 1])
    x11 = lerp(wx, w[0, 1, 1], w[1, 1, 1])
    return lerp(wz, lerp(wy, x00, x10), lerp(wy, x01, x11)).astype(np.float32)


def fbm_full(pts, omega, octaves):
    """fBm with zero ray differentials, i.e. all `octaves` octaves, lambda *= 1.99 per octave."""
    pts = np.asarray(pts, np.float32)
    s = np.zeros(pts.shape[0], np.float32)
    lam, o = np.float32(1), np.float32(1)
    for _ in range(octaves):
        s += o * perlin(pts * lam)
        lam = np.float32(lam * np.float32(1.99))
        o = np.float32(o * np.float32(omega))
    return s


# ----------------------------------------------------------------------------- scenes

CAMERA_BOX = "0 0 3.5\t0 0 0\t0 1 0\t40\t3.5\n"
IDENTITY_SUBJECT = "0 0 0\t0 1 0\t0\t1\n"


def _box_meshes(d):
    # open front (camera side, +z); walls face inward
    write_quads(os.path.join(d, "box_white.bin"), [
        ((-1, -1, -1), (0, 0, 2), (2, 0, 0)),   # floor y=-1, normal +y
        ((-1, 1, -1), (2, 0, 0), (0, 0, 2)),    # ceiling y=+1, normal -y
        ((-1, -1, -1), (2, 0, 0), (0, 2, 0)),   # back z=-1, normal +z
    ])
    write_quads(os.path.join(d, "box_red.bin"), [((-1, -1, -1), (0, 2, 0), (0, 0, 2))])    # x=-1, +x
    write_quads(os.path.join(d, "box_green.bin"), [((1, -1, -1), (0, 0, 2), (0, 2, 0))])   # x=+1, -x
    write_quads(os.path.join(d, "box_light.bin"), [((-0.25, 0.999, -0.25), (0.5, 0, 0), (0, 0, 0.5))])  # -y


def _box_scene_text(meshes_extra=""):
    return (CAMERA_BOX + IDENTITY_SUBJECT + "0\n"
            "4\tbox_white\tbox_red\tbox_green\tbox_light\n"
            "4\n"
            "L\tc\t0.7 0.7 0.7\t0\n"
            "L\tc\t0.7 0.1 0.1\t0\n"
            "L\tc\t0.1 0.7 0.1\t0\n"
            "L\tc\t0 0 0\t0\n"
            "1\t10 10 10\n"
            "0\n")


def write_box_sphere(d, level=4):
    """Writes box.scene + sphere.subject (+ meshes) into directory d; returns (scene, subject)
    names relative to d, as app.params would list them."""
    os.makedirs(d, exist_ok=True)
    _box_meshes(d)
    v, f = icosphere(level)
    write_bin(os.path.join(d, "sphere.bin"), v * 0.5, v, f, f)
    with open(os.path.join(d, "box.scene"), "w") as fh:
        fh.write(_box_scene_text())
    with open(os.path.join(d, "sphere.subject"), "w") as fh:
        fh.write("0\n1\tsphere\n1\nL\tc\t0.8 0.8 0.8\t0\n")
    return "box", "sphere"


def write_tri_light_box(d, level=3, facing_up=False):
    """The box + icosphere scene with its ceiling light as one triangle (the path tracer's light
    choice never picks the last light, a reference quirk that is exact with one light, so the path
    tracer and bidirectional path tracing estimate the same image); returns (scene, subject).
    facing_up: the triangle hangs at y = 0.9 and emits toward the ceiling, which then lights the
    room indirectly (next-event estimation from the room never sees its emitting side)."""
    os.makedirs(d, exist_ok=True)
    _box_meshes(d)
    if facing_up:
        p = np.array([(-0.3, 0.9, -0.3), (0.3, 0.9, -0.3), (0.0, 0.9, 0.3)])
        write_bin(os.path.join(d, "tri_light.bin"), p, np.array([(0.0, 1.0, 0.0)]), np.array([[0, 2, 1]]),
                  np.zeros((1, 3), np.int64))
    else:
        p = np.array([(-0.3, 0.999, -0.3), (0.3, 0.999, -0.3), (0.0, 0.999, 0.3)])
        write_bin(os.path.join(d, "tri_light.bin"), p, np.array([(0.0, -1.0, 0.0)]), np.array([[0, 2, 1]]),
                  np.zeros((1, 3), np.int64))
    v, f = icosphere(level)
    write_bin(os.path.join(d, "sphere.bin"), v * 0.5, v, f, f)
    text = _box_scene_text().replace("box_light", "tri_light").replace("1\t10 10 10\n", "1\t12 12 12\n")
    with open(os.path.join(d, "tribox.scene"), "w") as fh:
        fh.write(text)
    with open(os.path.join(d, "sphere.subject"), "w") as fh:
        fh.write("0\n1\tsphere\n1\nL\tc\t0.8 0.8 0.8\t0\n")
    return "tribox", "sphere"


# Point lights of the point-light scene: world position, intensity (the `pointLights` grammar
# extension of the loader; the reference has a PointLight but no file syntax for it).
POINT_LIGHTS = [((-0.6, 0.55, 0.35), (1.6, 1.2, 0.8)), ((0.55, -0.45, 0.5), (0.4, 0.8, 1.6))]


def write_point_lights(d, level=3):
    """The box + icosphere scene lit by the ceiling light, two point lights (POINT_LIGHTS) and a
    constant infinite light of 0.1 through the open front.  Lights in table order: the two
    ceiling triangles, the point lights, the infinite light (the reference's NEE never picks the
    last light, so every point light is sampled)."""
    os.makedirs(d, exist_ok=True)
    _box_meshes(d)
    v, f = icosphere(level)
    write_bin(os.path.join(d, "sphere.bin"), v * 0.5, v, f, f)
    text = _box_scene_text()
    assert text.endswith("0\n")
    text = text[:-2] + "1\t0.1 0.1 0.1\n" + "pointLights\t%d\n" % len(POINT_LIGHTS) + "".join(
        "%g %g %g\t%g %g %g\n" % (*p, *i) for p, i in POINT_LIGHTS)
    with open(os.path.join(d, "points.scene"), "w") as fh:
        fh.write(text)
    with open(os.path.join(d, "sphere.subject"), "w") as fh:
        fh.write("0\n1\tsphere\n1\nL\tc\t0.8 0.8 0.8\t0\n")
    return "points", "sphere"


def with_camera(d, scene, view, name):
    """Writes d/name.scene: `scene`'s file with its camera line replaced by a view's camera (a dict
    with frm, at, up, vfov, focus, as lts_render_views takes them), so that lts_render and the FP64
    renderer draw what that view draws.  Returns name."""
    with open(os.path.join(d, scene + ".scene")) as fh:
        lines = fh.read().split("\n")
    up = view.get("up", (0, 1, 0))
    lines[0] = "%r %r %r\t%r %r %r\t%r %r %r\t%r\t%r" % (*map(float, view["frm"]), *map(float, view["at"]),
                                                      *map(float, up), float(view["vfov"]), float(view.get("focus", 1.0)))
    with open(os.path.join(d, name + ".scene"), "w") as fh:
        fh.write("\n".join(lines))
    return name


def write_displaced(d, level=8, amplitude=0.1, radius=0.5):
    """Box + level-`level` icosphere displaced by amplitude*fbm(8, 0.5), wrinkled Lambertian."""
    os.makedirs(d, exist_ok=True)
    _box_meshes(d)
    v, f = icosphere(level)
    p = (v * radius).astype(np.float32)
    disp = fbm_full(p * np.float32(4.0), 0.5, 8).astype(np.float64)
    pos = v * (radius + amplitude * disp)[:, None]
    write_bin(os.path.join(d, "displaced.bin"), pos, v, f, f)
    with open(os.path.join(d, "box.scene"), "w") as fh:
        fh.write(_box_scene_text())
    with open(os.path.join(d, "displaced.subject"), "w") as fh:
        fh.write("0\n1\tdisplaced\n1\nL\tw\t8 0.5\t0\n")
    return "box", "displaced"


def uv_sphere(rings, segs):
    """Unit lat-long sphere: vertices (float64) and triangles; fans at the poles, two triangles
    per quad elsewhere: 2 * segs * (rings - 1) triangles, counter-clockwise seen from outside."""
    th = np.pi * np.arange(1, rings) / rings                      # interior rings
    ph = 2 * np.pi * np.arange(segs) / segs
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    ring = np.stack([st * np.cos(ph)[None, :], np.broadcast_to(ct, (rings - 1, segs)),
                     st * np.sin(ph)[None, :]], axis=-1).reshape(-1, 3)
    v = np.concatenate([[[0.0, 1.0, 0.0]], ring, [[0.0, -1.0, 0.0]]])
    top, bot = 0, v.shape[0] - 1
    idx = 1 + np.arange((rings - 1) * segs).reshape(rings - 1, segs)
    nxt = np.roll(idx, -1, axis=1)
    f = [np.stack([np.full(segs, top), nxt[0], idx[0]], axis=1)]
    a, b, c, d = idx[:-1], nxt[:-1], nxt[1:], idx[1:]
    f.append(np.stack([a, b, c], axis=-1).reshape(-1, 3))
    f.append(np.stack([a, c, d], axis=-1).reshape(-1, 3))
    f.append(np.stack([np.full(segs, bot), idx[-1], nxt[-1]], axis=1))
    return v, np.concatenate(f).astype(np.int64)


STRESS_SPHERE = (256, 512)   # rings, segments: 261,120 triangles per sphere


def write_stress_scene(d, rings=STRESS_SPHERE[0], segs=STRESS_SPHERE[1], copies=8, seed=2, amplitude=0.1,
                       instanced=False):
    """The material and divergence stress scene (see the module docstring); smaller `rings` and
    `segs` give the same layout with coarser spheres (parity cases).  instanced: the conductor
    spheres are `copies` instances of one unit-sphere file (the loader's `instances` record:
    mesh entry, translation, scale), written as stress_inst.scene / stress_inst.subject; their
    world triangles are the file's scaled and moved in float32, so they differ from the plain
    scene's by rounding."""
    os.makedirs(d, exist_ok=True)
    write_quads(os.path.join(d, "s_back.bin"), [((-1, -1, -1), (2, 0, 0), (0, 2, 0)),
                                                  ((-1, 1, -1), (2, 0, 0), (0, 0, 2))])
    write_quads(os.path.join(d, "s_floor.bin"), [((-1, -1, -1), (0, 0, 2), (2, 0, 0))])
    write_quads(os.path.join(d, "box_red.bin"), [((-1, -1, -1), (0, 2, 0), (0, 0, 2))])
    write_quads(os.path.join(d, "box_green.bin"), [((1, -1, -1), (0, 0, 2), (0, 2, 0))])
    write_quads(os.path.join(d, "box_light.bin"), [((-0.25, 0.999, -0.25), (0.5, 0, 0), (0, 0, 0.5))])
    v, f = uv_sphere(rings, segs)
    glass_c, glass_r = np.array([0.0, -0.55, 0.0]), 0.35
    disp = fbm_full((v * glass_r).astype(np.float32) * np.float32(4.0), 0.5, 8).astype(np.float64)
    write_bin(os.path.join(d, "glass.bin"), glass_c + v * (glass_r + amplitude * disp)[:, None], v, f, f)
    rng = np.random.default_rng(seed)
    r = 0.14
    centres, alphas = [], []
    while len(centres) < copies:
        c = rng.uniform([-0.8, -0.85, -0.8], [0.8, 0.7, 0.6])
        if np.linalg.norm(c - glass_c) < glass_r + amplitude + r + 0.02:
            continue
        if any(np.linalg.norm(c - o) < 2 * r + 0.02 for o in centres):
            continue
        centres.append(c)
        alphas.append(float(rng.uniform(0.05, 0.5)))
    names = []
    if instanced:
        write_bin(os.path.join(d, "unit_sphere.bin"), v, v, f, f)
        names = ["unit_sphere"] * copies
    else:
        for k, c in enumerate(centres):
            names.append(f"metal{k}")
            write_bin(os.path.join(d, f"metal{k}.bin"), c + v * r, v, f, f)
    name = "stress_inst" if instanced else "stress"
    inst = ""
    if instanced:  # subject meshes come first in the mesh order: glass is 0, the spheres 1 ..
        inst = "instances\t%d\n" % copies + "".join(
            "%d\t%r %r %r\t%r\n" % (1 + k, *map(float, c), float(r)) for k, c in enumerate(centres))
    with open(os.path.join(d, name + ".scene"), "w") as fh:
        fh.write(CAMERA_BOX + IDENTITY_SUBJECT + "0\n"
                 "5\ts_back\ts_floor\tbox_red\tbox_green\tbox_light\n"
                 "5\n"
                 "L\tc\t0.7 0.7 0.7\t0\n"
                 "L\tm\t8 0.5 4 1\t0\n"
                 "L\tc\t0.7 0.1 0.1\t0\n"
                 "L\tc\t0.1 0.7 0.1\t0\n"
                 "L\tc\t0 0 0\t0\n"
                 "1\t10 10 10\n"
                 "1\t0.5 0.5 0.5\n" + inst)
    with open(os.path.join(d, name + ".subject"), "w") as fh:
        fh.write("0\n%d\tglass\t%s\n%d\n" % (1 + copies, "\t".join(names), 1 + copies))
        fh.write("G\tc\t1 1 1\tc\t1 1 1\t1.5\n")
        for a in alphas:
            fh.write("C\tc\t3.9 2.4 1.8\tc\t0.2 0.4 1.4\t%.6f\n" % a)
    return name, name


def random_triangles(n, seed=1):
    """(n, 3, 3) float32 vertices: centroids U[0,1)^3, vertices centroid + N(0,1e-3)^3."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3), dtype=np.float32)
    e = rng.standard_normal((n, 3, 3), dtype=np.float32) * np.float32(1e-3)
    return (c + e).astype(np.float32) + np.float32(0.0)


def write_random_tris(d, n, seed=1):
    """random_triangles as a single-mesh subject inside an otherwise empty scene."""
    os.makedirs(d, exist_ok=True)
    t = random_triangles(n, seed)
    p = t.reshape(-1, 3)
    idx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    nrm = np.array([[0, 0, 1]], np.float32)
    write_bin(os.path.join(d, "rand.bin"), p, nrm, idx, np.zeros_like(idx))
    with open(os.path.join(d, "rand.scene"), "w") as fh:
        fh.write(CAMERA_BOX + IDENTITY_SUBJECT + "0\n0\n0\n0\n0\n")
    with open(os.path.join(d, "rand.subject"), "w") as fh:
        fh.write("0\n1\trand\n1\nL\tc\t0.5 0.5 0.5\t0\n")
    return "rand", "rand"


def write_app_params(path, width, height, spp, bounces, rr, fmt, output, scene, subject):
    """app.params: 9 whitespace-separated tokens (FileIO.cuh:234-257)."""
    with open(path, "w") as fh:
        fh.write(f"{width} {height}\n{spp}\n{bounces}\n{rr}\n{fmt}\n{output}\n{scene}\n{subject}\n")


def write_materials_scene(d, level=3):
    """Parity workload exercising the non-Lambertian paths the reference can load: a glass
    icosphere (eta 1.5) on the left, a mirror icosphere on the right, Oren-Nayar walls
    (sigma 20 deg), a marble-textured floor, fBm and wrinkled side walls, the ceiling area light
    and a constant infinite light (0.5) seen through the open front."""
    os.makedirs(d, exist_ok=True)
    write_quads(os.path.join(d, "m_back.bin"), [((-1, -1, -1), (2, 0, 0), (0, 2, 0)),
                                                  ((-1, 1, -1), (2, 0, 0), (0, 0, 2))])
    write_quads(os.path.join(d, "m_floor.bin"), [((-1, -1, -1), (0, 0, 2), (2, 0, 0))])
    write_quads(os.path.join(d, "m_left.bin"), [((-1, -1, -1), (0, 2, 0), (0, 0, 2))])
    write_quads(os.path.join(d, "m_right.bin"), [((1, -1, -1), (0, 0, 2), (0, 2, 0))])
    write_quads(os.path.join(d, "box_light.bin"), [((-0.25, 0.999, -0.25), (0.5, 0, 0), (0, 0, 0.5))])
    v, f = icosphere(level)
    write_bin(os.path.join(d, "glass.bin"), v * 0.35 + np.array([-0.4, -0.6, 0.1]), v, f, f)
    write_bin(os.path.join(d, "mirror.bin"), v * 0.3 + np.array([0.45, -0.65, -0.3]), v, f, f)
    with open(os.path.join(d, "materials.scene"), "w") as fh:
        fh.write(CAMERA_BOX + IDENTITY_SUBJECT + "0\n"
                 "5\tm_back\tm_floor\tm_left\tm_right\tbox_light\n"
                 "5\n"
                 "L\tc\t0.7 0.7 0.7\t20\n"
                 "L\tm\t8 0.5 4 1\t0\n"
                 "L\tf\t8 0.5\t0\n"
                 "L\tw\t8 0.5\t10\n"
                 "L\tc\t0 0 0\t0\n"
                 "1\t10 10 10\n"
                 "1\t0.5 0.5 0.5\n")
    with open(os.path.join(d, "spheres.subject"), "w") as fh:
        fh.write("0\n2\tglass\tmirror\n2\nG\tc\t1 1 1\tc\t1 1 1\t1.5\nR\tc\t0.9 0.9 0.9\t0\n")
    return "materials", "spheres"
