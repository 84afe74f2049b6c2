"""GB300 (sm_103a) renderer for the hot path of tierChampion/LightTransportSimulation.

The compute path is the in-tree CUDA library `_lib/liblts_gb300.so` behind the C-ABI of
`include/lts_capi.h`; this module is a thin ctypes layer over it that mirrors the reference's
host-side interfaces:

  read_application_parameters(path)          core/FileIO.cuh:234-257
  Scene.parse(root, scene, subject, w, h)    core/SceneLoader.cuh:195-360 (parseScene)
  Scene.create_bvh_tree(mode)                acceleration/BVH.cuh:411-452 (CreateBVHTree)
  PathTracingIntegrator(max_bounce, rr_start, scene).render(spp, seed)
                                             intergrators/PathTracingIntegrator.cuh:18-109
  write_image(path, rgb, format)             core/ImageO.cuh:16-78

There is no CPU fallback: without the compiled library, or without a GPU, the calls raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblts_gb300.so")

LTS_OK = 0
ERRORS = {1: "LTS_ERR_ARG", 2: "LTS_ERR_IO", 3: "LTS_ERR_PARSE", 4: "LTS_ERR_CUDA", 5: "LTS_ERR_OOM",
          6: "LTS_ERR_UNSUPPORTED", 7: "LTS_ERR_STATE", 8: "LTS_ERR_DEVICE"}
BVH_REFERENCE = 0
BVH_SORTED = 1
INTEGRATOR_MEGAKERNEL = 0
INTEGRATOR_WAVEFRONT = 1
INTEGRATOR_FP64 = 2
INTEGRATOR_BDPT = 3

# Every symbol include/lts_capi.h declares.
EXPORTS = ["lts_create", "lts_destroy", "lts_last_error", "lts_stream", "lts_read_app_params", "lts_load_scene",
           "lts_scene_info_get", "lts_scene_get_triangles", "lts_scene_get_camera",
           "lts_scene_get_light_distribution", "lts_bvh_build", "lts_bvh_build_triangles",
           "lts_bvh_build_device_async", "lts_bvh_dump_get", "lts_render", "lts_render_async", "lts_film_get",
           "lts_write_image", "lts_get_metrics", "lts_bvh_build_noalloc", "lts_debug_trace_sample",
           "lts_debug_trace_get", "lts_set_option", "lts_debug_umma_probe", "lts_mlp_init", "lts_mlp_set_params",
           "lts_mlp_get_params", "lts_mlp_forward", "lts_mlp_train_step", "lts_mlp_forward_device_async",
           "lts_mlp_train_step_device_async", "lts_render_views", "lts_autotune_views", "lts_obj_to_bin",
           "lts_debug_wait_timeout", "lts_debug_kat", "lts_intersect", "lts_scene_get_image",
           "lts_debug_image_lookup"]


class LtsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class AppParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("spp", ctypes.c_int32),
                ("max_bounce", ctypes.c_int32), ("rr_start", ctypes.c_int32), ("format", ctypes.c_int32),
                ("output", ctypes.c_char * 256), ("scene", ctypes.c_char * 256), ("subject", ctypes.c_char * 256)]


class SceneInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("triangles", "meshes", "subject_meshes", "materials", "lights",
                                               "area_light_meshes", "has_infinite", "width", "height",
                                               "max_mesh_triangles", "instances", "prototypes", "images")]


class BvhDump(ctypes.Structure):
    _fields_ = [("sorted_codes", ctypes.c_void_p), ("sorted_ids", ctypes.c_void_p), ("node_key", ctypes.c_void_p),
                ("node_left", ctypes.c_void_p), ("node_right", ctypes.c_void_p), ("node_bounds", ctypes.c_void_p)]


class RenderDesc(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_int32), ("max_bounce", ctypes.c_int32), ("rr_start", ctypes.c_int32),
                ("seed", ctypes.c_uint32), ("integrator", ctypes.c_int32), ("x0", ctypes.c_int32),
                ("y0", ctypes.c_int32), ("x1", ctypes.c_int32), ("y1", ctypes.c_int32),
                ("record_samples", ctypes.c_int32), ("bvh_mode", ctypes.c_int32)]


class RenderOut(ctypes.Structure):
    _fields_ = [("film_rgb", ctypes.c_void_p), ("film_sums", ctypes.c_void_p), ("sample_L", ctypes.c_void_p),
                ("sample_sig", ctypes.c_void_p), ("render_ms", ctypes.c_double), ("rays", ctypes.c_double),
                ("node_visits", ctypes.c_double), ("tri_tests", ctypes.c_double)]


class Metrics(ctypes.Structure):
    _fields_ = [("bvh_build_ms", ctypes.c_double), ("bvh_stage_ms", ctypes.c_double * 5),
                ("render_ms", ctypes.c_double), ("paths", ctypes.c_double), ("rays", ctypes.c_double),
                ("device_bytes", ctypes.c_int64), ("kernel_launches", ctypes.c_int32),
                ("render_launches", ctypes.c_int32), ("render_iterations", ctypes.c_int32),
                ("render_stage_ms", ctypes.c_double * 6), ("kind_rays", ctypes.c_double * 3),
                ("kind_node_visits", ctypes.c_double * 3), ("kind_tri_tests", ctypes.c_double * 3),
                ("cache_queries", ctypes.c_double), ("cache_train_samples", ctypes.c_int32),
                ("cache_train_loss", ctypes.c_double), ("cache_bias", ctypes.c_double),
                ("cache_train_ms", ctypes.c_double), ("scene_parse_ms", ctypes.c_double),
                ("scene_upload_ms", ctypes.c_double), ("render_bvh_ms", ctypes.c_double),
                ("scene_upload_bytes", ctypes.c_int64), ("render_bvh_bytes", ctypes.c_int64),
                ("render_two_level", ctypes.c_int32)]


_lib = None


def library():
    """Loads the compiled renderer; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with lighttransportsimulation_gb300.build.build()")
        lib = ctypes.CDLL(LIB_PATH)
        P, I, V = ctypes.c_void_p, ctypes.c_int32, None
        sig = {
            "lts_create": (I, [ctypes.POINTER(P), I]), "lts_destroy": (V, [P]),
            "lts_last_error": (ctypes.c_char_p, [P]), "lts_stream": (P, [P]),
            "lts_read_app_params": (I, [ctypes.c_char_p, ctypes.POINTER(AppParams)]),
            "lts_load_scene": (I, [P, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, I, I]),
            "lts_scene_info_get": (I, [P, ctypes.POINTER(SceneInfo)]),
            "lts_scene_get_triangles": (I, [P, P]), "lts_scene_get_camera": (I, [P, P]),
            "lts_scene_get_light_distribution": (I, [P, P, P]),
            "lts_bvh_build": (I, [P, I, ctypes.POINTER(BvhDump)]),
            "lts_bvh_build_triangles": (I, [P, P, I, I, I, ctypes.POINTER(BvhDump)]),
            "lts_bvh_build_device_async": (I, [P, P, I, I, I]),
            "lts_bvh_dump_get": (I, [P, ctypes.POINTER(BvhDump)]),
            "lts_render": (I, [P, ctypes.POINTER(RenderDesc), ctypes.POINTER(RenderOut)]),
            "lts_render_async": (I, [P, ctypes.POINTER(RenderDesc)]),
            "lts_film_get": (I, [P, P, P]),
            "lts_write_image": (I, [ctypes.c_char_p, P, I, I, I]),
            "lts_get_metrics": (I, [P, ctypes.POINTER(Metrics)]),
            "lts_bvh_build_noalloc": (I, [P, I, I, I, P, P, P, P, P, P]),
            "lts_debug_trace_sample": (I, [P, ctypes.c_int64]),
            "lts_debug_trace_get": (I, [P, P]),
            "lts_set_option": (I, [P, ctypes.c_char_p, ctypes.c_int64]),
            "lts_debug_umma_probe": (I, [P, I, I, P, P, P]),
            "lts_mlp_init": (I, [P, ctypes.c_uint32]),
            "lts_mlp_set_params": (I, [P, P]),
            "lts_mlp_get_params": (I, [P, P]),
            "lts_mlp_forward": (I, [P, P, I, P]),
            "lts_mlp_train_step": (I, [P, P, P, I, ctypes.c_float, P, P]),
            "lts_mlp_forward_device_async": (I, [P, P, I, P]),
            "lts_obj_to_bin": (I, [ctypes.c_char_p]),
            "lts_mlp_train_step_device_async": (I, [P, P, P, I, ctypes.c_float, P]),
            "lts_render_views": (I, [P, P, I, ctypes.POINTER(RenderDesc), P, ctypes.POINTER(RenderOut)]),
            "lts_autotune_views": (I, [P, P, I, ctypes.POINTER(RenderDesc), P]),
            "lts_debug_wait_timeout": (I, [P, I]),
            "lts_debug_kat": (I, [P, I, P, I, P]),
            "lts_intersect": (I, [P, P, I, I, P, P]),
            "lts_scene_get_image": (I, [P, I, I, P, P]),
            "lts_debug_image_lookup": (I, [P, I, P, I, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Context:
    """One renderer context (lts_create / lts_destroy).  device=-1: host-only (parsing)."""

    def __init__(self, device=0):
        self.lib = library()
        h = ctypes.c_void_p()
        rc = self.lib.lts_create(ctypes.byref(h), device)
        if rc != LTS_OK:
            raise LtsError(rc, "lts_create failed (no CUDA device or driver)" if device >= 0 else "lts_create")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.lts_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        if rc != LTS_OK:
            raise LtsError(rc, self.lib.lts_last_error(self.h).decode())

    def stream(self):
        return self.lib.lts_stream(self.h)

    def set_option(self, key, value):
        """Wavefront tuning knobs ("wavefront_pool", "wavefront_sample_chunk"); needs a loaded scene."""
        self.check(self.lib.lts_set_option(self.h, key.encode(), int(value)))

    def metrics(self):
        m = Metrics()
        self.check(self.lib.lts_get_metrics(self.h, ctypes.byref(m)))
        return m


def read_application_parameters(path):
    """app.params -> dict (width, height, spp, max_bounce, rr_start, format, output, scene, subject)."""
    p = AppParams()
    rc = library().lts_read_app_params(path.encode(), ctypes.byref(p))
    if rc != LTS_OK:
        raise LtsError(rc, path)
    d = {f: getattr(p, f) for f, _ in AppParams._fields_}
    for k in ("output", "scene", "subject"):
        d[k] = d[k].decode()
    return d


class Scene:
    """Scene{intersect, simpleIntersect, lights, lightCount} (acceleration/Scene.cuh:10-33) as
    device tables owned by a Context; parse() replaces parseScene."""

    def __init__(self, ctx):
        self.ctx = ctx

    @classmethod
    def parse(cls, ctx, root, scene, subject, width, height):
        root = os.path.join(root, "")
        ctx.check(ctx.lib.lts_load_scene(ctx.h, root.encode(), scene.encode(),
                                         (subject or "").encode(), width, height))
        s = cls(ctx)
        s.info = s.query_info()
        return s

    def query_info(self):
        i = SceneInfo()
        self.ctx.check(self.ctx.lib.lts_scene_info_get(self.ctx.h, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in SceneInfo._fields_}

    @property
    def light_count(self):
        return self.info["lights"]

    def triangles(self):
        out = np.empty(self.info["triangles"] * 9, np.float32)
        self.ctx.check(self.ctx.lib.lts_scene_get_triangles(self.ctx.h, _ptr(out)))
        return out.reshape(-1, 3, 3)

    def camera(self):
        out = np.empty(23, np.float32)
        self.ctx.check(self.ctx.lib.lts_scene_get_camera(self.ctx.h, _ptr(out)))
        return out

    def light_distribution(self):
        n = self.info["lights"]
        func = np.empty(max(n, 1), np.float32)
        cdf = np.empty(n + 1, np.float32)
        self.ctx.check(self.ctx.lib.lts_scene_get_light_distribution(self.ctx.h, _ptr(func), _ptr(cdf)))
        return func[:n], cdf

    def _query(self, o, d, tmax, any_hit):
        o = np.asarray(o, np.float32).reshape(-1, 3)
        d = np.asarray(d, np.float32).reshape(-1, 3)
        n = len(o)
        rays = np.zeros((n, 8), np.float32)
        rays[:, 0:3], rays[:, 4:7] = o, d
        rays[:, 3] = np.broadcast_to(np.asarray(tmax, np.float32), (n,))
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        self.ctx.check(self.ctx.lib.lts_intersect(self.ctx.h, _ptr(rays), n, 1 if any_hit else 0, _ptr(prim), _ptr(t)))
        return prim, t

    def intersect(self, o, d, tmax=np.inf):
        """Scene::intersect (acceleration/Scene.cuh:26-29) over a batch of rays: the closest hit's
        primitive in scene order (-1: none) and distance."""
        return self._query(o, d, tmax, False)

    def simple_intersect(self, o, d, tmax):
        """Scene::simpleIntersect (acceleration/Scene.cuh:30-32): True where a hit lies before tmax."""
        return self._query(o, d, tmax, True)[0] == 1

    def image(self, index, level=0):
        """Level `level` of image texture `index` (the fixed mode's pyramid): (h, w, 3) float32,
        row 0 the bottom row, and the image's level count."""
        wh = np.zeros(3, np.int32)
        self.ctx.check(self.ctx.lib.lts_scene_get_image(self.ctx.h, index, level, _ptr(wh), None))
        out = np.empty(int(wh[0]) * int(wh[1]) * 3, np.float32)
        self.ctx.check(self.ctx.lib.lts_scene_get_image(self.ctx.h, index, level, _ptr(wh), _ptr(out)))
        return out.reshape(int(wh[1]), int(wh[0]), 3), int(wh[2])

    def image_lookup(self, index, st):
        """Mipmap::lookUp of image texture `index` on the device at (n, 2) texture coordinates."""
        st = np.ascontiguousarray(st, np.float32).reshape(-1, 2)
        out = np.empty((len(st), 3), np.float32)
        self.ctx.check(self.ctx.lib.lts_debug_image_lookup(self.ctx.h, index, _ptr(st), len(st), _ptr(out)))
        return out

    def create_bvh_tree(self, mode=BVH_SORTED, dump=True):
        """LBVH of the scene; returns the dump dict (codes, ids, node arrays) when dump."""
        n = self.info["triangles"]
        arrays, d = _dump_arrays(n) if dump else (None, None)
        self.ctx.check(self.ctx.lib.lts_bvh_build(self.ctx.h, mode, ctypes.byref(d) if dump else None))
        return arrays


def _dump_arrays(n):
    nodes = 2 * n - 1
    a = {"sorted_codes": np.empty(n, np.uint32), "sorted_ids": np.empty(n, np.int32),
         "node_key": np.empty(nodes, np.int32), "node_left": np.empty(nodes, np.int32),
         "node_right": np.empty(nodes, np.int32), "node_bounds": np.empty(nodes * 6, np.float32)}
    d = BvhDump(*[a[f].ctypes.data for f, _ in BvhDump._fields_])
    return a, d


def build_bvh_triangles(ctx, tris, mode=BVH_SORTED, code_limit=-1):
    """LBVH over an (n, 3, 3) float32 triangle soup; returns the dump dict."""
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    arrays, d = _dump_arrays(tris.shape[0])
    ctx.check(ctx.lib.lts_bvh_build_triangles(ctx.h, _ptr(tris), tris.shape[0], mode, code_limit, ctypes.byref(d)))
    return arrays


class PathTracingIntegrator:
    """PathTracingIntegrator(maxBounce, rrStart, camera, sampler, scene) and its evaluate()
    over the film (intergrators/PathTracingIntegrator.cuh:18-109); the camera and the Gaussian
    filter come from the parsed scene, the sampler from (spp, seed)."""

    def __init__(self, max_bounce, rr_start, scene, integrator=INTEGRATOR_MEGAKERNEL, bvh_mode=BVH_SORTED):
        self.max_bounce, self.rr_start, self.scene = max_bounce, rr_start, scene
        self.integrator, self.bvh_mode = integrator, bvh_mode

    def desc(self, spp, seed, crop=None, record=False):
        x0, y0, x1, y1 = crop if crop is not None else (0, 0, 0, 0)
        return RenderDesc(spp, self.max_bounce, self.rr_start, seed, self.integrator, x0, y0, x1, y1,
                          1 if record else 0, self.bvh_mode)

    def render(self, spp, seed, crop=None, record=False, film=True, sums=False):
        info = self.scene.info
        W, H = info["width"], info["height"]
        d = self.desc(spp, seed, crop, record)
        cw = (crop[2] - crop[0]) if crop else W
        ch = (crop[3] - crop[1]) if crop else H
        res = {}
        rgb = np.empty(W * H * 3, np.float32) if film else None
        fs = np.empty(W * H * 4, np.float64) if sums else None
        L = np.empty(cw * ch * spp * 3, np.float32) if record else None
        sig = np.empty(cw * ch * spp, np.uint64) if record else None
        o = RenderOut(rgb.ctypes.data if film else None, fs.ctypes.data if sums else None,
                      L.ctypes.data if record else None, sig.ctypes.data if record else None, 0.0, 0.0, 0.0, 0.0)
        ctx = self.scene.ctx
        ctx.check(ctx.lib.lts_render(ctx.h, ctypes.byref(d), ctypes.byref(o)))
        if film:
            res["film"] = rgb.reshape(H, W, 3)
        if sums:
            res["film_sums"] = fs.reshape(H, W, 4)
        if record:
            res["L"] = L.reshape(ch, cw, spp, 3)
            res["sig"] = sig.reshape(ch, cw, spp)
        res["render_ms"] = o.render_ms
        res["rays"] = o.rays
        res["node_visits"] = o.node_visits
        res["tri_tests"] = o.tri_tests
        return res


def obj_to_bin(mesh_name):
    """mesh_name.obj -> mesh_name.bin in the reference's binary mesh layout (lts_obj_to_bin)."""
    rc = library().lts_obj_to_bin(str(mesh_name).encode())
    if rc != LTS_OK:
        raise LtsError(rc, str(mesh_name))


def write_image(path, rgb, fmt):
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w = rgb.shape[:2]
    rc = library().lts_write_image(path.encode(), _ptr(rgb), w, h, fmt)
    if rc != LTS_OK:
        raise LtsError(rc, path)


class RadianceCacheMLP:
    """The radiance-cache network of a context (lts_mlp_*): 96 bf16 features -> RGB."""

    PARAMS = 23552
    FEATURES = 96

    def __init__(self, ctx, seed=1):
        self.ctx = ctx
        ctx.check(ctx.lib.lts_mlp_init(ctx.h, seed))

    def params(self):
        import numpy as np
        out = np.zeros(self.PARAMS, np.float32)
        self.ctx.check(self.ctx.lib.lts_mlp_get_params(self.ctx.h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_params(self, p):
        import numpy as np
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.PARAMS
        self.ctx.check(self.ctx.lib.lts_mlp_set_params(self.ctx.h, p.ctypes.data_as(ctypes.c_void_p)))

    def forward(self, feat_bits):
        import numpy as np
        f = np.ascontiguousarray(feat_bits, np.uint16).reshape(-1, self.FEATURES)
        out = np.zeros((f.shape[0], 3), np.float32)
        self.ctx.check(self.ctx.lib.lts_mlp_forward(self.ctx.h, f.ctypes.data_as(ctypes.c_void_p), f.shape[0],
                                                    out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def train_step(self, feat_bits, targets, lr, want_grad=False):
        """Returns (loss, gradient before the update or None)."""
        import numpy as np
        f = np.ascontiguousarray(feat_bits, np.uint16).reshape(-1, self.FEATURES)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 3)
        loss = ctypes.c_float()
        g = np.zeros(self.PARAMS, np.float32) if want_grad else None
        self.ctx.check(self.ctx.lib.lts_mlp_train_step(
            self.ctx.h, f.ctypes.data_as(ctypes.c_void_p), t.ctypes.data_as(ctypes.c_void_p), f.shape[0],
            ctypes.c_float(lr), ctypes.byref(loss), g.ctypes.data_as(ctypes.c_void_p) if want_grad else None))
        return loss.value, g


    def forward_device_async(self, d_features, n, d_out):
        """Inference on device buffers (bf16 feature bits, FP32 RGB out), on the context's stream."""
        self.ctx.check(self.ctx.lib.lts_mlp_forward_device_async(self.ctx.h, ctypes.c_void_p(d_features), int(n),
                                                                 ctypes.c_void_p(d_out)))

    def train_step_device_async(self, d_features, d_targets, n, lr, d_loss=None):
        """One training pass (and Adam step when lr > 0) on device buffers, on the context's stream."""
        self.ctx.check(self.ctx.lib.lts_mlp_train_step_device_async(
            self.ctx.h, ctypes.c_void_p(d_features), ctypes.c_void_p(d_targets), int(n), ctypes.c_float(lr),
            ctypes.c_void_p(d_loss) if d_loss else None))


class View(ctypes.Structure):
    """One camera of a batched render (lts_view): the scene file's camera record fields plus film
    size, samples per pixel and seed."""
    _fields_ = [("frm", ctypes.c_float * 3), ("at", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("vfov", ctypes.c_float), ("focus", ctypes.c_float), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("spp", ctypes.c_int32), ("seed", ctypes.c_uint32)]


class AutotuneResult(ctypes.Structure):
    _fields_ = [("pool_log2", ctypes.c_int32), ("trace_blocks_per_sm", ctypes.c_int32), ("graph", ctypes.c_int32),
                ("ms_default", ctypes.c_double), ("ms_best", ctypes.c_double)]


def _view_array(views):
    arr = (View * len(views))()
    for k, v in enumerate(views):
        arr[k].frm[:] = v["frm"]
        arr[k].at[:] = v["at"]
        arr[k].up[:] = v.get("up", (0, 1, 0))
        arr[k].vfov = v["vfov"]
        arr[k].focus = v.get("focus", 1.0)
        arr[k].width, arr[k].height, arr[k].spp, arr[k].seed = v["width"], v["height"], v["spp"], v["seed"]
    return arr


def autotune_views(scene, views, max_bounce, rr_start, bvh_mode=1):
    """lts_autotune_views: picks and sets the wavefront's pool size, trace grid and graph mode for
    this batch of views; returns the choice as a dict."""
    ctx = scene.ctx
    desc = RenderDesc()
    desc.spp, desc.max_bounce, desc.rr_start, desc.integrator, desc.bvh_mode = 1, max_bounce, rr_start, 1, bvh_mode
    res = AutotuneResult()
    ctx.check(ctx.lib.lts_autotune_views(ctx.h, _view_array(views), len(views), ctypes.byref(desc), ctypes.byref(res)))
    return {"pool_log2": res.pool_log2, "trace_blocks_per_sm": res.trace_blocks_per_sm, "graph": res.graph,
            "ms_default": res.ms_default, "ms_best": res.ms_best}


def render_views(scene, views, max_bounce, rr_start, bvh_mode=1):
    """Renders every view (dicts with frm, at, up, vfov, focus, width, height, spp, seed) of the
    loaded scene in batched wavefront launches; returns ([H x W x 3 images, flipped like
    lts_render's film], render_ms)."""
    import numpy as np
    ctx = scene.ctx
    n = len(views)
    arr = _view_array(views)
    films = [np.zeros(v["width"] * v["height"] * 3, np.float32) for v in views]
    ptrs = (ctypes.c_void_p * n)(*[f.ctypes.data for f in films])
    desc = RenderDesc()
    desc.spp, desc.max_bounce, desc.rr_start, desc.integrator, desc.bvh_mode = 1, max_bounce, rr_start, 1, bvh_mode
    out = RenderOut()
    ctx.check(ctx.lib.lts_render_views(ctx.h, arr, n, ctypes.byref(desc), ptrs, ctypes.byref(out)))
    return [f.reshape(v["height"], v["width"], 3) for f, v in zip(films, views)], out.render_ms
