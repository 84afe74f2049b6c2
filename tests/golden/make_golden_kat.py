"""Regenerates tests/golden/kat_reference.npz: known-answer vectors of single functions, computed
by the reference's own code (oracle/_ref/lts_ref kat -- tierChampion/LightTransportSimulation's
sources compiled for the host by oracle/ref/build_ref.sh).

Functions and record layouts are the LTS_KAT_* of include/lts_capi.h: the Trowbridge-Reitz
distribution (D, Lambda, G1, G, Pdf, the visible-normal sampling of Sample11 / sampleWH), the
conductor microfacet BRDF (MicrofacetReflection f / Pdf / sampleF with FresnelConductor), the
dielectric and conductor Fresnel terms, improved Perlin noise, fbm, turbulence, offsetRayOrigin
and quakeIIIFastInvSqrt.  Inputs are seeded (numpy, seed 8) and drawn to cover each function's
branches: both hemispheres, grazing and normal incidence, the dielectric's swapped clamp
(cosines beyond +-1), the Sample11 normal-incidence branch, fractional and full octave counts.
Records of G1, G and Pdf are isotropic (alphaX == alphaY: the renderers' conductor is isotropic).

Usage (from the repository root): oracle/ref/build_ref.sh && python tests/golden/make_golden_kat.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.path.join(ROOT, "oracle", "_ref", "lts_ref")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat_reference.npz")
N = 512

# LTS_KAT_* of include/lts_capi.h
FUNCS = {"quake_rsqrt": 0, "fresnel_dielectric": 1, "fresnel_conductor": 2, "tr_d": 3, "tr_lambda": 4, "tr_g1": 5,
         "tr_g": 6, "tr_sample11": 7, "tr_sample_wh": 8, "tr_pdf": 9, "mf_f": 10, "mf_pdf": 11, "mf_sample": 12,
         "perlin": 13, "fbm": 14, "turbulence": 15, "offset_origin": 16}


def unit(rng, n, upper=None):
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    if upper is True:
        v[:, 2] = np.abs(v[:, 2])
    return v


def inputs(rng):
    """Seeded input records (n x 16 float32) per function."""
    rec = {}
    z = lambda: np.zeros((N, 16))  # noqa: E731
    a = z()
    a[:, 0] = 10.0 ** rng.uniform(-6, 6, N)
    a[:16, 0] = [1, 2, 4, 8, 16, 64, 256, 1024, 4096, 65536, 0.5, 0.25, 3, 10, 100, 1e-3]
    rec["quake_rsqrt"] = a
    a = z()
    a[:, 0] = rng.uniform(-1.2, 1.2, N)
    a[:, 1] = np.where(rng.random(N) < 0.5, 1.0, rng.uniform(1.0, 2.5, N))
    a[:, 2] = np.where(rng.random(N) < 0.5, 1.5, rng.uniform(1.0, 2.5, N))
    rec["fresnel_dielectric"] = a
    a = z()
    a[:, 0] = rng.uniform(-1, 1, N)
    a[:, 1:4] = rng.uniform(0.1, 4.0, (N, 3))
    a[:, 4:7] = rng.uniform(0.0, 5.0, (N, 3))
    rec["fresnel_conductor"] = a
    alpha = lambda: rng.uniform(0.05, 0.5, N)  # noqa: E731
    for name in ("tr_d", "tr_lambda"):
        a = z()
        a[:, 0:3] = unit(rng, N)
        a[:, 3] = alpha()
        a[:, 4] = np.where(rng.random(N) < 0.5, a[:, 3], alpha())
        rec[name] = a
    a = z()
    a[:, 0:3] = unit(rng, N)
    a[:, 3] = a[:, 4] = alpha()
    rec["tr_g1"] = a
    a = z()
    a[:, 0:3], a[:, 3:6] = unit(rng, N), unit(rng, N)
    a[:, 6] = a[:, 7] = alpha()
    rec["tr_g"] = a
    a = z()
    a[:, 0] = np.where(rng.random(N) < 0.1, rng.uniform(0.99995, 1.0, N), rng.uniform(0.02, 0.9999, N))
    a[:, 1:3] = rng.uniform(0.0, 1.0, (N, 2))
    rec["tr_sample11"] = a
    a = z()
    a[:, 0:3] = unit(rng, N)
    a[:, 3] = alpha()
    a[:, 4] = np.where(rng.random(N) < 0.5, a[:, 3], alpha())
    a[:, 5:7] = rng.uniform(0.0, 1.0, (N, 2))
    rec["tr_sample_wh"] = a
    a = z()
    a[:, 0:3], a[:, 3:6] = unit(rng, N, upper=True), unit(rng, N, upper=True)
    a[:, 6] = a[:, 7] = alpha()
    rec["tr_pdf"] = a
    a = z()
    a[:, 0:3], a[:, 3:6] = unit(rng, N, upper=True), unit(rng, N, upper=True)
    a[:, 6] = alpha()
    a[:, 7:10] = rng.uniform(0.5, 1.0, (N, 3))
    a[:, 10:13] = rng.uniform(0.1, 4.0, (N, 3))
    a[:, 13:16] = rng.uniform(0.0, 5.0, (N, 3))
    rec["mf_f"] = a
    a = z()
    a[:, 0:3], a[:, 3:6] = unit(rng, N, upper=True), unit(rng, N)
    a[:, 6] = alpha()
    rec["mf_pdf"] = a
    a = z()
    a[:, 0:3] = unit(rng, N, upper=True)
    a[:, 3] = alpha()
    a[:, 4:6] = rng.uniform(0.0, 1.0, (N, 2))
    a[:, 6:9] = rng.uniform(0.5, 1.0, (N, 3))
    a[:, 9:12] = rng.uniform(0.1, 4.0, (N, 3))
    a[:, 12:15] = rng.uniform(0.0, 5.0, (N, 3))
    rec["mf_sample"] = a
    a = z()
    a[:, 0:3] = np.where(rng.random((N, 1)) < 0.5, rng.uniform(-2, 2, (N, 3)), rng.uniform(-60, 60, (N, 3)))
    rec["perlin"] = a
    for name in ("fbm", "turbulence"):
        a = z()
        a[:, 0:3] = rng.uniform(-5, 5, (N, 3))
        scale = np.where(rng.random(N) < 0.3, 0.0, 10.0 ** rng.uniform(-4, 0, N))[:, None]
        a[:, 3:6] = rng.standard_normal((N, 3)) * scale
        a[:, 6:9] = rng.standard_normal((N, 3)) * scale
        a[:, 9] = rng.uniform(0.3, 0.7, N)
        a[:, 10] = rng.integers(1, 9, N)
        rec[name] = a
    a = z()
    a[:, 0:3] = rng.uniform(-10, 10, (N, 3))
    a[:, 3:6] = 10.0 ** rng.uniform(-7, -3, (N, 3))
    a[:, 6:9] = unit(rng, N)
    a[:, 9:12] = unit(rng, N)
    rec["offset_origin"] = a
    return {k: v.astype(np.float32) for k, v in rec.items()}


def run(exe, fn, a):
    with tempfile.TemporaryDirectory() as td:
        i, o = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        a.astype(np.float32).tofile(i)
        subprocess.run([exe, "kat", str(fn), i, o], check=True)
        return np.fromfile(o, np.float32).reshape(-1, 16)


def main():
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/lts_ref is missing: run oracle/ref/build_ref.sh first")
    rec = inputs(np.random.default_rng(8))
    out = {}
    for name, a in rec.items():
        out[f"in_{name}"] = a
        out[f"out_{name}"] = run(REF, FUNCS[name], a)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
