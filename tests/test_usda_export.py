"""USD (ASCII) export without pxr: the layer has the prims of the reference's
renderer (utils/renderer.py:8-122) and the points of every rendered frame as
time samples (CPU test with host arrays)."""
import numpy as np


class _Field:
    def __init__(self, a):
        self.a = a

    def to_numpy(self):
        return self.a.copy()


def test_usda_layer_roundtrip(tmp_path):
    from xpbd_gpu.usda import USDMeshRenderer, read_usda_points
    rng = np.random.default_rng(0)
    pts = rng.normal(size=(7, 3)).astype(np.float32)
    field = _Field(pts)
    faces = _Field(np.array([0, 1, 2, 2, 3, 4, 4, 5, 6], dtype=np.uint32))
    path = str(tmp_path / "out" / "run.usdc")
    r = USDMeshRenderer(path, 3, 60, use_binary=True, root_prim_path="root")
    r.add_dynamic_mesh(field, faces, "deformable_mesh")
    r.add_static_sphere([0.5, 0.3, 0.5], 0.3, name="sdf_sphere_1")
    r.add_static_cube([0.5, 0.15, 0.5], [0.4, 0.3, 0.4], name="sdf_cube_2")
    r.add_static_plane([0, 0, 0], [0, 2, 0], extent=4.0, name="sdf_plane_0")
    frames = []
    for k in range(4):  # the fourth render is past totalframes and ignored
        field.a = (pts + 0.1 * k).astype(np.float32)
        frames.append(field.a.copy())
        r.render()
    r.save()
    r.close()
    assert r.filepath.endswith(".usda") and r.get_file_size_mb() > 0
    text = open(r.filepath).read()
    assert text.startswith("#usda 1.0")
    assert 'defaultPrim = "root"' in text and 'upAxis = "Y"' in text and "endTimeCode = 3" in text
    for token in ('def Xform "root"', 'def Mesh "deformable_mesh"', 'def Sphere "sdf_sphere_1"',
                  'def Cube "sdf_cube_2"', 'def Mesh "sdf_plane_0"', "int[] faceVertexCounts = [3, 3, 3]",
                  "int[] faceVertexIndices = [0, 1, 2, 2, 3, 4, 4, 5, 6]", "double radius = 0.3"):
        assert token in text, token
    samples = read_usda_points(r.filepath)
    assert sorted(samples) == [1, 2, 3]
    for t in (1, 2, 3):
        np.testing.assert_allclose(samples[t], frames[t - 1], rtol=1e-7, atol=1e-7)
    plane = text[text.index('def Mesh "sdf_plane_0"'):]
    assert "(2, 0, -2)" in plane.replace("-0,", "0,") or "(-2, 0, -2)" in plane.replace("-0,", "0,")
