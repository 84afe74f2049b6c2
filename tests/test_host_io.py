"""Host I/O against the reference's own converter and writers (golden fixtures made by
tests/golden/make_golden_io.py from oracle/_ref/lts_ref): OBJ -> .bin conversion
(core/FileIO.cuh:20-45, 73-164), scenes whose meshes are OBJ files (parseMesh, FileIO.cuh:213-232)
and the PPM / PFM film writers (core/ImageO.cuh:16-78).  CPU only."""
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN

IO = os.path.join(GOLDEN, "io")


@pytest.mark.parametrize("name", ["sphere_a", "sphere_b"])
def test_obj_to_bin_matches_the_reference(built_lib, tmp_path, name):
    import lighttransportsimulation_gb300 as lts
    shutil.copy(os.path.join(IO, name + ".obj"), tmp_path / (name + ".obj"))
    lts.obj_to_bin(str(tmp_path / name))
    assert (tmp_path / (name + ".bin")).read_bytes() == open(os.path.join(IO, name + ".bin"), "rb").read()


def _obj_scene(d):
    from lighttransportsimulation_gb300 import scenes
    z = np.load(os.path.join(IO, "obj_scene.npz"))
    scenes._box_meshes(d)
    with open(os.path.join(d, "box.scene"), "w") as fh:
        fh.write(scenes._box_scene_text().replace(scenes.IDENTITY_SUBJECT, str(z["subject"]), 1))
    with open(os.path.join(d, "spheres.subject"), "w") as fh:
        fh.write("0\n2\tsphere_a\tsphere_b\n2\nL\tc\t0.8 0.8 0.8\t0\nL\tc\t0.5 0.6 0.7\t0\n")
    for name in ("sphere_a", "sphere_b"):
        shutil.copy(os.path.join(IO, name + ".obj"), os.path.join(d, name + ".obj"))
    return z["tri_p"]


def test_scene_with_obj_meshes_matches_the_reference(built_lib, tmp_path):
    """Meshes given only as .obj load to the reference's world triangles (bit patterns), and the
    loader leaves the reference's .bin conversions beside them; a second load reads those."""
    import lighttransportsimulation_gb300 as lts
    d = str(tmp_path)
    tri_ref = _obj_scene(d)
    for _ in range(2):
        ctx = lts.Context(-1)
        s = lts.Scene.parse(ctx, d, "box", "spheres", 64, 64)
        assert np.array_equal(s.triangles().reshape(-1).view(np.uint32), tri_ref.view(np.uint32))
        for name in ("sphere_a", "sphere_b"):
            assert (tmp_path / (name + ".bin")).read_bytes() == open(os.path.join(IO, name + ".bin"), "rb").read()
        ctx.close()


@pytest.mark.parametrize("fmt,ext", [(0, "ppm"), (1, "pfm")])
def test_image_writers_match_the_reference(built_lib, tmp_path, fmt, ext):
    import lighttransportsimulation_gb300 as lts
    film = np.fromfile(os.path.join(IO, "film_in.f32"), np.float32).reshape(5, 7, 3)
    out = tmp_path / ("film." + ext)
    lts.write_image(str(out), film, fmt)
    assert out.read_bytes() == open(os.path.join(IO, "film." + ext), "rb").read()


@pytest.mark.parametrize("text,code", [
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n", 0),      # smallest valid mesh
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", 3),                         # corner without uv / n fields
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf //1 2//1 3//1\n", 3),       # no position index
    ("v 0 zero 0\n", 3),                                                 # stof rejects the token
    ("v 0 0 0\nv 1 0\n", 3),                                             # file ends inside a vertex
    ("vn 0 0 1\nf 1//1 2//1\n", 3),                                      # file ends inside a face
])
def test_obj_reader_edges(built_lib, tmp_path, text, code):
    """The reader's accepted input, and a parse error where the reference has no defined result."""
    import lighttransportsimulation_gb300 as lts
    (tmp_path / "m.obj").write_text(text)
    if code == 0:
        lts.obj_to_bin(str(tmp_path / "m"))
        from lighttransportsimulation_gb300 import scenes
        p, uv, n, idx = scenes.read_bin(str(tmp_path / "m.bin"))
        assert p.shape == (3, 3) and uv.shape == (0, 2) and n.shape == (1, 3)
        assert idx.tolist() == [[[0, 0, 0], [1, 0, 0], [2, 0, 0]]]
    else:
        with pytest.raises(lts.LtsError) as e:
            lts.obj_to_bin(str(tmp_path / "m"))
        assert e.value.code == code


def test_missing_mesh_is_an_io_error(built_lib, tmp_path):
    import lighttransportsimulation_gb300 as lts
    with pytest.raises(lts.LtsError) as e:
        lts.obj_to_bin(str(tmp_path / "absent"))
    assert e.value.code == 2
