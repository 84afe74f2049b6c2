/*
 * lts_render_app -- the thin host program that replaces the reference's main
 * (src/LightTransportSimulation.cu:23-146): read app.params, parse the scene, build the LBVH,
 * render, write the image.  Plain C over the library's C-ABI (include/lts_capi.h); every step
 * returns a status instead of exiting inside the library.
 *
 *   lts_render_app ROOT [--device N] [--seed S] [--integrator megakernel|wavefront|fp64]
 *
 * ROOT is the directory holding app.params; the scene, subject and output paths in it are taken
 * relative to ROOT (the reference resolves them against its project directory).  The seed is an
 * argument (the reference seeds with time(0)).  --device -1 makes a host-only context: the scene
 * is parsed and summarised, and the render step reports that it needs a GPU (status 7).
 * Exit status: 0, or the LTS_ERR_* code of the step that failed.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/lts_capi.h"

static int usage(void) {
    fprintf(stderr, "usage: lts_render_app ROOT [--device N] [--seed S] [--integrator megakernel|wavefront|fp64]\n");
    return LTS_ERR_ARG;
}

int main(int argc, char** argv) {
    if (argc < 2) return usage();
    const char* root = argv[1];
    int device = 0, integrator = LTS_INTEGRATOR_MEGAKERNEL;
    uint32_t seed = 0;
    for (int i = 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--device") && i + 1 < argc) {
            device = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--seed") && i + 1 < argc) {
            seed = (uint32_t)strtoul(argv[++i], NULL, 10);
        } else if (!strcmp(argv[i], "--integrator") && i + 1 < argc) {
            const char* v = argv[++i];
            if (!strcmp(v, "megakernel")) integrator = LTS_INTEGRATOR_MEGAKERNEL;
            else if (!strcmp(v, "wavefront")) integrator = LTS_INTEGRATOR_WAVEFRONT;
            else if (!strcmp(v, "fp64")) integrator = LTS_INTEGRATOR_FP64;
            else return usage();
        } else {
            return usage();
        }
    }
    size_t rl = strlen(root);
    const char* sep = (rl > 0 && root[rl - 1] == '/') ? "" : "/";
    char path[4096], rootdir[4096], out_path[4096];
    snprintf(path, sizeof path, "%s%sapp.params", root, sep);
    snprintf(rootdir, sizeof rootdir, "%s%s", root, sep);

    /* readApplicationParameters (core/FileIO.cuh:234-257) */
    lts_app_params p;
    int rc = lts_read_app_params(path, &p);
    if (rc) {
        fprintf(stderr, "lts_render_app: cannot read %s (status %d)\n", path, rc);
        return rc;
    }
    /* device setup (LightTransportSimulation.cu:51-55) */
    lts_ctx* ctx = NULL;
    rc = lts_create(&ctx, device);
    if (rc) {
        fprintf(stderr, "lts_render_app: no context on device %d (status %d)\n", device, rc);
        return rc;
    }
    /* parseScene (core/SceneLoader.cuh:195-360) */
    rc = lts_load_scene(ctx, rootdir, p.scene, p.subject, p.width, p.height);
    if (!rc) {
        lts_scene_info info;
        rc = lts_scene_info_get(ctx, &info);
        if (!rc)
            printf("scene %s + %s: %d triangles, %d meshes, %d lights%s, %dx%d, %d spp, %d bounces\n", p.scene,
                   p.subject, info.triangles, info.meshes, info.lights, info.has_infinite ? " (one infinite)" : "",
                   p.width, p.height, p.spp, p.max_bounce);
    }
    /* PathTracingKernel (LightTransportSimulation.cu:103-110), the LBVH built on demand */
    float* rgb = NULL;
    if (!rc) {
        lts_render_desc d;
        memset(&d, 0, sizeof d);
        d.spp = p.spp;
        d.max_bounce = p.max_bounce;
        d.rr_start = p.rr_start;
        d.seed = seed;
        d.integrator = integrator;
        d.bvh_mode = LTS_BVH_SORTED;
        rgb = (float*)malloc(sizeof(float) * 3 * (size_t)p.width * (size_t)p.height);
        lts_render_out o;
        memset(&o, 0, sizeof o);
        o.film_rgb = rgb;
        rc = rgb ? lts_render(ctx, &d, &o) : LTS_ERR_OOM;
        if (!rc) printf("rendered in %.3f ms of device time, %.0f rays\n", o.render_ms, o.rays);
    }
    /* outputResultAndOpen -> writeToPPM / writeToPFM (Camera.cu:242-289, core/ImageO.cuh) */
    if (!rc) {
        snprintf(out_path, sizeof out_path, "%s%s", rootdir, p.output);
        rc = lts_write_image(out_path, rgb, p.width, p.height, p.format);
        if (!rc) printf("wrote %s\n", out_path);
    }
    if (rc) fprintf(stderr, "lts_render_app: status %d: %s\n", rc, lts_last_error(ctx));
    free(rgb);
    lts_destroy(ctx);
    return rc;
}
