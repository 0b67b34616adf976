"""Camera.gpuCamera (Scene/Camera.swift:167-218): the scalar float32 basis of
`Camera.gpu_camera` against a vectorised numpy float32 restatement of the same
operations, bit for bit, over seeded random cameras (perspective and
orthographic, up vectors parallel to the view direction, degenerate up and
view vectors), and the reference's own camera known answers (APITests.swift:23-76)."""
import math

import numpy as np
import pytest

from denrimrendererkit_gb300.scene import Camera

f32 = np.float32


def normalize_rows(v):
    v = v.astype(f32)
    inv = (f32(1.0) / np.sqrt((v * v).sum(axis=-1, dtype=f32))).astype(f32)
    return (v * inv[..., None]).astype(f32)


def reference_basis(cam: Camera, width: int, height: int):
    o = np.asarray(cam.origin, f32)
    vd = np.asarray(cam.target, f32) - o
    forward = normalize_rows(vd[None])[0] if float((vd * vd).sum()) > 1e-8 else np.array([0, 0, -1], f32)
    up = np.asarray(cam.up, f32)
    up = normalize_rows(up[None])[0] if float((up * up).sum()) > 1e-8 else np.array([0, 1, 0], f32)
    helper = up if abs(float(np.dot(forward, up))) < 0.999 else np.array([1, 0, 0], f32)
    right = normalize_rows(np.cross(forward, helper)[None])[0]
    true_up = np.cross(right, forward).astype(f32)
    aspect = f32(width) / f32(height)
    if cam.orthographic_scale is None:
        theta = f32(cam.vertical_field_of_view_degrees) * f32(math.pi) / f32(180)
        vh = f32(2) * f32(math.tan(theta / f32(2)))
    else:
        vh = f32(max(cam.orthographic_scale, 0.0001))
    vw = f32(aspect * vh)
    horizontal = (vw * right).astype(f32)
    vertical = (vh * true_up).astype(f32)
    pc = (o + forward) if cam.orthographic_scale is None else o
    lower_left = (pc - horizontal * f32(0.5) - vertical * f32(0.5)).astype(f32)
    return o, lower_left, horizontal, vertical


def as_array(v):
    return np.array([v.x, v.y, v.z], f32)


def test_scalar_camera_basis_equals_vectorised_restatement():
    rng = np.random.default_rng(11)
    cams = []
    for i in range(3000):
        o = rng.normal(0, 3, 3)
        t = o + rng.normal(0, 2, 3) * (10.0 ** rng.uniform(-3, 2))
        up = rng.normal(0, 1, 3)
        kind = i % 6
        if kind == 1:
            up = (t - o) * rng.uniform(0.1, 5)  # parallel to the view direction
        elif kind == 2:
            up = np.zeros(3)  # degenerate up
        elif kind == 3:
            t = o.copy()  # degenerate view vector
        cams.append(Camera(tuple(o), tuple(t), up=tuple(up), vertical_field_of_view_degrees=float(rng.uniform(5, 120)),
                           orthographic_scale=float(rng.uniform(0.01, 20)) if kind == 4 else None))
    for c in cams:
        w, h = int(rng.integers(1, 4096)), int(rng.integers(1, 4096))
        got = c.gpu_camera(w, h)
        o, ll, hz, vt = reference_basis(c, w, h)
        for a, b in ((got.origin, o), (got.lower_left, ll), (got.horizontal, hz), (got.vertical, vt)):
            assert as_array(a).view(np.uint32).tolist() == b.view(np.uint32).tolist(), c


def _length(v):
    return math.sqrt(v.x * v.x + v.y * v.y + v.z * v.z)


def test_perspective_camera_known_answer():
    # APITests.testPerspectiveCameraGeneratesPerspectiveGPUCamera (APITests.swift:23-37)
    gpu = Camera((0, 0, 3), (0, 0, 0), vertical_field_of_view_degrees=90).gpu_camera(200, 100)
    assert abs(gpu.origin.w - 0) < 1e-4 and abs(gpu.origin.z - 3) < 1e-4
    assert abs(gpu.lower_left.z - 2) < 1e-4
    assert abs(_length(gpu.horizontal) - 4) < 1e-4 and abs(_length(gpu.vertical) - 2) < 1e-4


def test_orthographic_camera_known_answer():
    # APITests.testOrthographicCameraGeneratesOrthographicGPUCamera (APITests.swift:39-55)
    gpu = Camera((0, 0, 3), (0, 0, 2), orthographic_scale=6).gpu_camera(200, 100)
    assert abs(gpu.origin.w - 1) < 1e-4 and abs(gpu.origin.z - 3) < 1e-4
    assert abs(gpu.lower_left.x + 6) < 1e-4 and abs(gpu.lower_left.y + 3) < 1e-4 and abs(gpu.lower_left.z - 3) < 1e-4
    assert abs(_length(gpu.horizontal) - 12) < 1e-4 and abs(_length(gpu.vertical) - 6) < 1e-4


def test_camera_lens_known_answer():
    # APITests.testCameraLensReachesGPUCamera (APITests.swift:57-67)
    gpu = Camera((0, 0, 3), (0, 0, 0), focus_distance=4.5, aperture_radius=0.08).gpu_camera(200, 100)
    assert abs(gpu.lens.x - 0.08) < 1e-4 and abs(gpu.lens.y - 4.5) < 1e-4


def test_camera_focused_on_point_known_answer():
    # APITests.testCameraFocusedOnPointSetsFocusDistance (APITests.swift:69-76)
    cam = Camera((0, 0, 5), (0, 0, 0)).focused((0, 0, 1), aperture_radius=0.12)
    assert abs(cam.focus_distance - 4) < 1e-4 and abs(cam.aperture_radius - 0.12) < 1e-4
    # behind the camera: the focal distance clamps at 0.0001; a coincident target looks down -z
    assert Camera((0, 0, 5), (0, 0, 0)).focused((0, 0, 9), 0.1).focus_distance == 0.0001
    assert Camera((1, 2, 3), (1, 2, 3)).focused((1, 2, 1), -1.0).focus_distance == pytest.approx(2.0)
    assert Camera((1, 2, 3), (1, 2, 3)).focused((1, 2, 1), -1.0).aperture_radius == 0.0
