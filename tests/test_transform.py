"""Instance transforms against the reference's own known answers
(TransformTests.swift:6-50).  Instances are materialised into the flat
triangle list here (no top-level instance tree is built), so the last test
checks the baked triangles and the instance's world bounds from them."""
import numpy as np

from denrimrendererkit_gb300 import Material, Mesh, RenderScene, Transform, compile_scene


def test_translation_moves_points():
    # TransformTests.testTranslationMovesPoints (:6-13)
    p = Transform.translation((2, 3, 4)).transform_points(np.array([[1, 1, 1]], np.float32))[0]
    assert np.allclose(p, [3, 4, 5], atol=1e-4)


def test_scale_transforms_normals_with_the_inverse_transpose():
    # TransformTests.testScaleTransformsNormalWithInverseTranspose (:15-22)
    n = np.array([[0, 2, 4]], np.float32)
    n /= np.linalg.norm(n)
    t = Transform.scale((1, 2, 4)).transform_normals(n)[0]
    assert abs(t[0]) < 1e-4 and abs(t[1] - t[2]) < 1e-4


def test_scene_compilation_bakes_the_instance_transform():
    # TransformTests.testSceneCompilationBakesInstanceTransform (:24-50)
    scene = RenderScene()
    m = scene.add_material(Material(base_color=(1, 1, 1)))
    scene.add(Mesh.quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)), m, Transform.translation((2, 0, 0)))
    build = compile_scene(scene)
    tris = build.triangles
    assert len(tris) == 2
    assert np.allclose([tris[0]["v0"][0], tris[0]["v1"][0], tris[0]["v2"][0]], [2, 3, 3], atol=1e-4)
    assert int(tris[0]["object_id"]) == 0
    xs = np.concatenate([tris[k][:, 0] for k in ("v0", "v1", "v2")])
    assert abs(xs.min() - 2) < 1e-4 and abs(xs.max() - 3) < 1e-4
    assert len(build.nodes) > 0
