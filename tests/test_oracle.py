"""CPU tests of the oracle itself: the project sampler against the published Philox KATs, and
(where the reference checkout is present) the committed fixtures against a fresh run of the
reference build."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "lts_ref")


def _philox_py(ctr, key):
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    M = 0xFFFFFFFF
    for _ in range(10):
        p0 = 0xD2511F53 * c0
        p1 = 0xCD9E8D57 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & M, p1 & M, ((p0 >> 32) ^ c3 ^ k1) & M, p0 & M
        k0 = (k0 + 0x9E3779B9) & M
        k1 = (k1 + 0xBB67AE85) & M
    return [c0, c1, c2, c3]


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    assert _philox_py([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    f = 0xFFFFFFFF
    assert _philox_py([f, f, f, f], [f, f]) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert _philox_py([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_c_sampler_matches_python(tmp_path):
    src = tmp_path / "s.c"
    src.write_text('#include <stdio.h>\n#include "lts_rng.h"\nint main(){for(unsigned k=0;k<8;++k)'
                   'printf("%.9g\\n",lts_rng_uniform(lts_rng_key(7u,1234u),3u,k));}\n')
    exe = tmp_path / "s"
    subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "oracle", "port"), str(src), "-o", str(exe)], check=True)
    got = [float(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]

    def wang(a):
        M = 0xFFFFFFFF
        a = (a ^ 61) ^ (a >> 16)
        a = (a + (a << 3)) & M
        a ^= a >> 4
        a = (a * 0x27D4EB2D) & M
        return a ^ (a >> 15)

    key = (7 + wang(1234)) & 0xFFFFFFFF
    want = [((_philox_py([k >> 2, 3, 0, 0], [key, 0x4C54530A])[k & 3] >> 8) + 1) / 16777216.0 for k in range(8)]
    np.testing.assert_array_equal(np.float32(got), np.float32(want))


@pytest.mark.skipif(not (os.path.exists(REF_BIN) and os.path.isdir("/root/reference/src")),
                    reason="reference build not available on this machine")
def test_fixtures_reproduce_from_reference(tmp_path):
    """The committed fixtures are exactly what the reference produces (regenerated here)."""
    import shutil
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    for f in os.listdir(GOLDEN):
        if f.endswith(".npz"):
            shutil.copy(os.path.join(GOLDEN, f), tmp_path / f)
    import make_golden_kat
    old, old_kat = make_golden.OUT, make_golden_kat.OUT
    try:
        make_golden.OUT = str(tmp_path)
        make_golden_kat.OUT = str(tmp_path / "kat_reference.npz")
        make_golden.main()
        make_golden.make_shipped("/root/reference")
        make_golden_kat.main()
    finally:
        make_golden.OUT, make_golden_kat.OUT = old, old_kat
    for f in os.listdir(GOLDEN):
        if not f.endswith(".npz"):
            continue
        a, b = np.load(os.path.join(GOLDEN, f)), np.load(tmp_path / f)
        for k in a.files:
            if k == "L" and f.startswith("render"):
                np.testing.assert_array_equal(a[k], b[k])
            else:
                assert np.array_equal(a[k], b[k]), (f, k)


def test_numpy_lbvh_matches_reference_fixture():
    """oracle/lbvh_np.py is pinned to the reference's own LBVH dumps."""
    from oracle import lbvh_np
    for kind in ("box_sphere", "materials"):
        fx = np.load(os.path.join(GOLDEN, f"lbvh_{kind}.npz"))
        tris = fx["tri_p"].reshape(-1, 3, 3)
        n = len(tris)
        # the reference codes ceil(maxMeshTris/16)*16 primitives; the largest mesh is the first
        # subject mesh in both scenes (5120 and 1280 triangles)
        limit = {"box_sphere": 5120, "materials": 1280}[kind]
        codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris, code_limit=limit))
        assert np.array_equal(codes, fx["sorted_codes"]) and np.array_equal(ids, fx["sorted_ids"])
        left, right = lbvh_np.karras_topology(codes)
        assert np.array_equal(left, fx["node_left"][: n - 1]) and np.array_equal(right, fx["node_right"][: n - 1])
        mn, mx = lbvh_np.tri_bounds(tris)
        lbvh_np.check_tree(fx["node_left"], fx["node_right"], fx["node_bounds"], np.concatenate([mn, mx], 1))


def _kat_run(exe, fn, a):
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        i, o = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        a.astype(np.float32).tofile(i)
        subprocess.run([exe, "kat", str(fn), i, o], check=True)
        return np.fromfile(o, np.float32).reshape(-1, 16)


KAT_FUNCS = {"quake_rsqrt": 0, "fresnel_dielectric": 1, "fresnel_conductor": 2, "tr_d": 3, "tr_lambda": 4,
             "tr_g1": 5, "tr_g": 6, "tr_sample11": 7, "tr_sample_wh": 8, "tr_pdf": 9, "mf_f": 10, "mf_pdf": 11,
             "mf_sample": 12, "perlin": 13, "fbm": 14, "turbulence": 15, "offset_origin": 16}


def kat_compare_mask(name, ref):
    """Output slots a comparison covers: all 16, except that a rejected microfacet sample
    (pdf 0) leaves wi unspecified (the reference writes it before rejecting, the others not)."""
    m = np.ones(ref.shape, bool)
    if name == "mf_sample":
        m[ref[:, 6] == 0, 0:3] = False
    return m


@pytest.mark.parametrize("name", list(KAT_FUNCS))
def test_port_matches_reference_known_answers(port_exe, name):
    """The port's restatement of each single function against the reference's own function
    (tests/golden/kat_reference.npz, made by oracle/_ref/lts_ref kat): bit for bit."""
    z = np.load(os.path.join(GOLDEN, "kat_reference.npz"))
    ref = z[f"out_{name}"]
    got = _kat_run(port_exe, KAT_FUNCS[name], z[f"in_{name}"])
    m = kat_compare_mask(name, ref)
    assert np.array_equal(got.view(np.uint32)[m], ref.view(np.uint32)[m])
