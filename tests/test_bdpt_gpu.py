"""Bidirectional path tracing (LTS_INTEGRATOR_BDPT) against the path tracer: both estimate the same
image, so their films of many samples agree up to Monte Carlo noise.  The reference's own BDPT is
disabled and unfinished (intergrators/BidirectionalPathIntegrator.cuh), so the path tracer -- held
per sample to the reference elsewhere -- is the oracle here.

The scenes keep to what both integrators estimate alike: one light triangle (the path tracer's
light choice never picks the last light, a reference quirk that is exact with one light),
constant textures (the path tracer evaluates textures with camera differentials, which light
paths do not have), no infinite light (unsupported by the bidirectional integrator), and no
glass: the reference's dielectric sends its Fresnel-reflected share straight on through the
surface (Specular.cuh:112) with the Fresnel term of the side the path arrives from, a
non-reciprocal BSDF, so light paths through it carry other weights than camera paths (measured:
the caustic under a glass ball 40 % dimmer in BDPT than in the path tracer, everything else
within noise).

Films are compared on 8 x 8 pixel blocks: the block means of BDPT and path tracer must differ by
no more than twice their combined seed-to-seed noise (measured: 0.9 to 1.0 times it)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAM = "0 0 3.5\t0 0 0\t0 1 0\t40\t3.5\n0 0 0\t0 1 0\t0\t1\n0\n"


def _tri_light(d):
    """The ceiling light as one triangle facing down."""
    from lighttransportsimulation_gb300 import scenes
    p = np.array([(-0.3, 0.999, -0.3), (0.3, 0.999, -0.3), (0.0, 0.999, 0.3)])
    scenes.write_bin(os.path.join(d, "tri_light.bin"), p, np.array([(0.0, -1.0, 0.0)]), np.array([[0, 2, 1]]),
                     np.zeros((1, 3), np.int64))


def _write(d, kind):
    from lighttransportsimulation_gb300 import scenes
    os.makedirs(d, exist_ok=True)
    scenes._box_meshes(d)
    _tri_light(d)
    v, f = scenes.icosphere(3)
    scenes.write_bin(os.path.join(d, "ball.bin"), v * 0.35 + np.array([-0.35, -0.65, 0.0]), v, f, f)
    scenes.write_bin(os.path.join(d, "ball2.bin"), v * 0.3 + np.array([0.45, -0.7, -0.3]), v, f, f)
    if kind == "diffuse":
        meshes = ["ball", "box_white", "box_red", "box_green", "tri_light"]
        mats = ["L\tc\t0.8 0.8 0.8\t0", "L\tc\t0.7 0.7 0.7\t0", "L\tc\t0.7 0.1 0.1\t0", "L\tc\t0.1 0.7 0.1\t0",
                "L\tc\t0 0 0\t0"]
        tail = "1\t12 12 12\n0\n"
    elif kind == "specular":  # mirror and rough conductor balls, Oren-Nayar walls, a conductor wall
        meshes = ["ball", "ball2", "box_white", "box_red", "box_green", "tri_light"]
        mats = ["R\tc\t0.9 0.9 0.9\t0", "C\tc\t3.9 2.4 1.8\tc\t0.2 0.4 1.4\t0.15", "L\tc\t0.7 0.7 0.7\t20",
                "C\tc\t3.9 2.4 1.8\tc\t0.2 0.4 1.4\t0.3", "L\tc\t0.1 0.7 0.1\t0", "L\tc\t0 0 0\t0"]
        tail = "1\t12 12 12\n0\n"
    else:  # point light only
        meshes = ["ball", "box_white", "box_red", "box_green"]
        mats = ["L\tc\t0.8 0.8 0.8\t0", "L\tc\t0.7 0.7 0.7\t0", "L\tc\t0.7 0.1 0.1\t0", "L\tc\t0.1 0.7 0.1\t0"]
        tail = "0\n0\npointLights\t1\n0.1 0.6 0.3\t2 2 2\n"
    text = CAM + "%d\t%s\n%d\n" % (len(meshes), "\t".join(meshes), len(mats)) + "\n".join(mats) + "\n" + tail
    open(os.path.join(d, kind + ".scene"), "w").write(text)
    return kind


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


def _blocks(img, b=8):
    h, w = img.shape[:2]
    return img[:h // b * b, :w // b * b].reshape(h // b, b, w // b, b, 3).mean(axis=(1, 3))


@pytest.mark.parametrize("kind", ["diffuse", "specular", "point"])
def test_bdpt_estimates_the_path_tracers_image(ctx, tmp_path, kind):
    import lighttransportsimulation_gb300 as lts
    d = str(tmp_path)
    sc = _write(d, kind)
    W = H = 96
    s = lts.Scene.parse(ctx, d, sc, "", W, H)
    maxb = 5
    pt = lts.PathTracingIntegrator(maxb, 3, s, integrator=lts.INTEGRATOR_MEGAKERNEL)
    bd = lts.PathTracingIntegrator(maxb, 3, s, integrator=lts.INTEGRATOR_BDPT)
    spp_pt, spp_bd = 4096, 512
    p1, p2 = (_blocks(pt.render(spp_pt, seed)["film"].astype(np.float64)) for seed in (1, 2))
    r1 = bd.render(spp_bd, 3)
    b1 = _blocks(r1["film"].astype(np.float64))
    b2 = _blocks(bd.render(spp_bd, 4)["film"].astype(np.float64))
    noise = np.sqrt(np.mean((p1 - p2) ** 2) / 2 + np.mean((b1 - b2) ** 2) / 2)
    diff = np.sqrt(np.mean((b1 - p1) ** 2))
    rel_mean = (b1.mean() - p1.mean()) / p1.mean()
    print(f"{kind}: image mean PT {p1.mean():.5f}, BDPT {b1.mean():.5f} ({rel_mean:+.4f}); block RMS BDPT - PT "
          f"{diff:.5f}, combined noise {noise:.5f}; BDPT {r1['render_ms']:.0f} ms for {spp_bd} spp")
    assert np.isfinite(b1).all() and p1.mean() > 0
    assert abs(rel_mean) < 0.01
    assert diff < 2.0 * noise + 1e-4


def test_bdpt_refuses_an_infinite_light(ctx, scene_dirs):
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["materials"]
    s = lts.Scene.parse(ctx, d, sc, sub, 32, 32)
    with pytest.raises(lts.LtsError):
        lts.PathTracingIntegrator(5, 3, s, integrator=lts.INTEGRATOR_BDPT).render(1, 1)
