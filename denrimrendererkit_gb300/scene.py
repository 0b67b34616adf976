"""Scene description and scene compile: the host side in front of the C ABI.

Python mirrors of the reference's public scene types and of the Swift host
code that turns a `RenderScene` into the POD arrays of an `AccelerationBuild`:

* `Mesh`, `Mesh.quad`, `Mesh.box`, `Mesh.gpu_triangles`
  (Sources/DenrimRendererKit/Geometry/Mesh.swift:4-186)
* `Transform` (Scene/Transform.swift:4-87)
* `Material` and its `gpu_material` packing (Scene/Material.swift:16-284)
* `Camera` and `gpu_camera` (Scene/Camera.swift:44-243)
* `Environment`, `Texture2D` (Scene/Environment.swift, Scene/Texture.swift)
* `RenderScene` (Scene/RenderScene.swift:73-860)
* `compile_scene`, the restatement of `LinearTriangleAccelerationBackend.build`
  (Acceleration/AccelerationBackend.swift:7-68): instance materialisation
  (InstanceAcceleration.swift:23-128), material/texture packing
  (MaterialGPUEncoding.swift:5-50), emissive-triangle light tagging and the
  flat BVH, both through the GB300 library's scene-compile helpers, and the
  environment importance table built on the GPU with an FP64 prefix sum.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

from . import abi

f32 = np.float32


def _normalize_rows(v: np.ndarray) -> np.ndarray:
    v = v.astype(f32)
    inv = (f32(1.0) / np.sqrt((v * v).sum(axis=-1, dtype=f32))).astype(f32)
    return (v * inv[..., None]).astype(f32)


def _dot3(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def _normalize3(v):
    inv = f32(1.0) / np.sqrt(_dot3(v, v))
    return (v[0] * inv, v[1] * inv, v[2] * inv)


def _cross3(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


# --------------------------------------------------------------- transform ---
@dataclasses.dataclass
class Transform:
    """Local-to-world 4x4 matrix (Scene/Transform.swift:4-87), row-major math matrix."""
    matrix: np.ndarray = dataclasses.field(default_factory=lambda: np.eye(4, dtype=f32))

    @staticmethod
    def identity() -> "Transform":
        return Transform()

    @staticmethod
    def translation(v) -> "Transform":
        m = np.eye(4, dtype=f32)
        m[:3, 3] = np.asarray(v, dtype=f32)
        return Transform(m)

    @staticmethod
    def scale(v) -> "Transform":
        m = np.eye(4, dtype=f32)
        m[0, 0], m[1, 1], m[2, 2] = (f32(x) for x in v)
        return Transform(m)

    @staticmethod
    def rotation_y(radians: float) -> "Transform":
        c, s = f32(math.cos(radians)), f32(math.sin(radians))
        m = np.eye(4, dtype=f32)
        m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
        return Transform(m)

    def __mul__(self, other: "Transform") -> "Transform":
        return Transform((self.matrix.astype(np.float64) @ other.matrix.astype(np.float64)).astype(f32))

    def is_identity(self) -> bool:
        return bool(np.array_equal(self.matrix, np.eye(4, dtype=f32)))

    def transform_points(self, p: np.ndarray) -> np.ndarray:
        m = self.matrix
        return (p @ m[:3, :3].T + m[:3, 3]).astype(f32)

    def transform_normals(self, n: np.ndarray) -> np.ndarray:
        inv_t = np.linalg.inv(self.matrix.astype(np.float64)).T.astype(f32)
        return _normalize_rows(n @ inv_t[:3, :3].T)


# -------------------------------------------------------------------- mesh ---
@dataclasses.dataclass
class Mesh:
    """Triangle mesh (Geometry/Mesh.swift:4-86)."""
    vertices: np.ndarray
    indices: np.ndarray
    normals: Optional[np.ndarray] = None
    texcoords: Optional[np.ndarray] = None

    @staticmethod
    def quad(a, b, c, d) -> "Mesh":
        """Mesh.quad (Mesh.swift:32-50)."""
        return Mesh(np.array([a, b, c, d], dtype=f32), np.array([0, 1, 2, 0, 2, 3], dtype=np.uint32),
                    texcoords=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=f32))

    @staticmethod
    def box(minimum=None, maximum=None, *, size=None) -> "Mesh":
        """Mesh.box(minimum:maximum:) (Mesh.swift:61-86); with `size` instead,
        Mesh.box(size:) (:52-58), the box of that size centred on the origin."""
        if size is not None:
            half = np.asarray(size, f32) * f32(0.5)
            minimum, maximum = -half, half
        lo, hi = np.asarray(minimum, f32), np.asarray(maximum, f32)
        v = np.array([[lo[0], lo[1], lo[2]], [hi[0], lo[1], lo[2]], [hi[0], hi[1], lo[2]], [lo[0], hi[1], lo[2]],
                      [lo[0], lo[1], hi[2]], [hi[0], lo[1], hi[2]], [hi[0], hi[1], hi[2]], [lo[0], hi[1], hi[2]]], f32)
        i = np.array([0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 4, 7, 0, 7, 3, 1, 2, 6, 1, 6, 5,
                      3, 7, 6, 3, 6, 2, 0, 1, 5, 0, 5, 4], np.uint32)
        return Mesh(v, i)

    def gpu_triangles(self, material_id: int = 0, transform: Optional[Transform] = None,
                      object_id: int = 0) -> np.ndarray:
        """Mesh.gpuTriangles (Mesh.swift:88-186): positions, vertex normals with
        the face-normal fallback, UVs and the UV tangent frame per triangle."""
        transform = transform or Transform.identity()
        idx = self.indices.reshape(-1, 3).astype(np.int64)
        n = idx.shape[0]
        out = np.zeros(n, dtype=abi.TRIANGLE_DTYPE)
        if n == 0:
            return out
        p = self.vertices.astype(f32)
        p0, p1, p2 = p[idx[:, 0]], p[idx[:, 1]], p[idx[:, 2]]
        if self.texcoords is not None and len(self.texcoords):
            tc = np.zeros((len(p), 2), f32)
            tc[: len(self.texcoords)] = self.texcoords
        else:
            tc = np.zeros((len(p), 2), f32)
        uv0, uv1, uv2 = tc[idx[:, 0]], tc[idx[:, 1]], tc[idx[:, 2]]
        e1, e2 = (p1 - p0).astype(f32), (p2 - p0).astype(f32)
        local_normal = _normalize_rows(np.cross(e1, e2))

        def vertex_normal(k):
            if self.normals is None or len(self.normals) == 0:
                return local_normal
            nn = np.zeros((len(p), 3), f32)
            valid = np.zeros(len(p), bool)
            m = min(len(self.normals), len(p))
            nn[:m] = self.normals[:m]
            valid[:m] = True
            vn = nn[idx[:, k]]
            ok = valid[idx[:, k]] & ((vn * vn).sum(-1) > 1e-8)
            res = local_normal.copy()
            res[ok] = _normalize_rows(vn[ok])
            return res

        normals = [vertex_normal(k) for k in range(3)]
        # tangentFrame (Mesh.swift:156-186)
        d1, d2 = (uv1 - uv0).astype(f32), (uv2 - uv0).astype(f32)
        den = (d1[:, 0] * d2[:, 1] - d2[:, 0] * d1[:, 1]).astype(f32)
        ok = np.abs(den) > 1e-6
        helper = np.where((np.abs(local_normal[:, 1]) < 0.999)[:, None], np.array([0, 1, 0], f32),
                          np.array([1, 0, 0], f32)).astype(f32)
        t_fb = _normalize_rows(np.cross(helper, local_normal))
        b_fb = np.cross(local_normal, t_fb).astype(f32)
        with np.errstate(divide="ignore", invalid="ignore"):
            fac = (f32(1) / np.where(ok, den, f32(1))).astype(f32)
            t_uv = _normalize_rows(fac[:, None] * (d2[:, 1:2] * e1 - d1[:, 1:2] * e2))
            b_uv = _normalize_rows(fac[:, None] * (-d2[:, 0:1] * e1 + d1[:, 0:1] * e2))
        tangent = np.where(ok[:, None], t_uv, t_fb)
        bitangent = np.where(ok[:, None], b_uv, b_fb)
        if not transform.is_identity():
            p0, p1, p2 = (transform.transform_points(x) for x in (p0, p1, p2))
        normals = [transform.transform_normals(x) for x in normals]
        tangent = transform.transform_normals(tangent)
        bitangent = transform.transform_normals(bitangent)
        for name, arr in (("v0", p0), ("v1", p1), ("v2", p2), ("n0", normals[0]), ("n1", normals[1]),
                          ("n2", normals[2]), ("tangent", tangent), ("bitangent", bitangent)):
            out[name][:, :3] = arr
        out["uv0"][:, :2], out["uv1"][:, :2], out["uv2"][:, :2] = uv0, uv1, uv2
        out["material_id"] = material_id
        out["object_id"] = object_id
        out["primitive_id"] = np.arange(n, dtype=np.uint32)
        return out


def icosphere(subdivisions: int, radius: float = 1.0) -> Mesh:
    """Subdivided icosahedron (20 * 4**subdivisions triangles) with smooth
    vertex normals.  The reference has no sphere-mesh generator; its scene
    builders only make quads and boxes, so this deterministic generator supplies
    the sphere geometry of the small and large benchmark scenes."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(faces, dtype=np.int64)
    for _ in range(subdivisions):
        edges = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
        uniq, inv = np.unique(edges, axis=0, return_inverse=True)
        mids = v[uniq[:, 0]] + v[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mids])
        nf = len(f)
        a = inv[:nf] + base
        b = inv[nf:2 * nf] + base
        c = inv[2 * nf:] + base
        f = np.concatenate([np.stack([f[:, 0], a, c], 1), np.stack([f[:, 1], b, a], 1),
                            np.stack([f[:, 2], c, b], 1), np.stack([a, b, c], 1)])
    return Mesh((v * radius).astype(f32), f.reshape(-1).astype(np.uint32), normals=v.astype(f32))


# ---------------------------------------------------------------- material ---
@dataclasses.dataclass
class Material:
    """Material (Scene/Material.swift:16-219) with the same defaults."""
    base_color: Sequence[float] = (0.8, 0.8, 0.8)
    emission: Sequence[float] = (0.0, 0.0, 0.0)
    emission_strength: float = 0.0
    roughness: float = 0.5
    metallic: float = 0.0
    specular: float = 1.0
    specular_color: Sequence[float] = (1.0, 1.0, 1.0)
    index_of_refraction: float = 1.5
    specular_anisotropy: float = 0.0
    clearcoat: float = 0.0
    clearcoat_color: Sequence[float] = (1.0, 1.0, 1.0)
    clearcoat_attenuation_color: Optional[Sequence[float]] = None
    clearcoat_thickness: float = 0.0
    clearcoat_roughness: float = 0.1
    clearcoat_index_of_refraction: float = 1.5
    thin_film: float = 0.0
    thin_film_thickness_nanometers: float = 450.0
    thin_film_index_of_refraction: float = 1.45
    sheen: float = 0.0
    sheen_color: Sequence[float] = (1.0, 1.0, 1.0)
    sheen_roughness: float = 0.5
    subsurface: float = 0.0
    subsurface_color: Optional[Sequence[float]] = None
    subsurface_radius: Sequence[float] = (1.0, 1.0, 1.0)
    subsurface_scale: float = 1.0
    subsurface_anisotropy: float = 0.0
    opacity: float = 1.0
    transmission: float = 0.0
    transmission_color: Optional[Sequence[float]] = None
    transmission_roughness: Optional[float] = None
    transmission_index_of_refraction: Optional[float] = None
    transmission_absorption_color: Sequence[float] = (1.0, 1.0, 1.0)
    transmission_absorption_distance: float = 0.0
    thin_walled: bool = False
    volume_scattering: float = 0.0
    volume_scattering_color: Optional[Sequence[float]] = None
    volume_scattering_distance: float = 1.0
    volume_anisotropy: float = 0.0
    base_color_texture: Optional["Texture2D"] = None
    normal_map: Optional["Texture2D"] = None

    def gpu_material(self, base_color_texture_index: Optional[int] = None,
                     normal_map_index: Optional[int] = None) -> np.ndarray:
        """Material.gpuMaterial (Material.swift:222-284)."""
        bc = tuple(self.base_color)
        sub_c = tuple(self.subsurface_color) if self.subsurface_color is not None else bc
        tr_c = tuple(self.transmission_color) if self.transmission_color is not None else bc
        tr_r = self.transmission_roughness if self.transmission_roughness is not None else self.roughness
        tr_ior = (self.transmission_index_of_refraction if self.transmission_index_of_refraction is not None
                  else self.index_of_refraction)
        vs_c = (tuple(self.volume_scattering_color) if self.volume_scattering_color is not None else
                (tuple(self.transmission_color) if self.transmission_color is not None else bc))
        cc_att = (tuple(self.clearcoat_attenuation_color) if self.clearcoat_attenuation_color is not None
                  else tuple(self.clearcoat_color))
        em = tuple(f32(e) * f32(self.emission_strength) for e in self.emission)
        m = np.zeros((), dtype=abi.MATERIAL_DTYPE)
        m["base_color"] = (*bc, self.opacity)
        m["emission"] = (*em, self.transmission)
        m["parameters"] = (self.roughness, self.metallic, float((base_color_texture_index if base_color_texture_index
                                                                   is not None else -1) + 1),
                           float((normal_map_index if normal_map_index is not None else -1) + 1))
        m["parameters2"] = (self.specular, self.index_of_refraction, self.clearcoat, self.clearcoat_roughness)
        m["specular_color"] = (*tuple(self.specular_color), self.clearcoat_index_of_refraction)
        m["sheen_color"] = (*tuple(self.sheen_color), self.sheen)
        m["transmission_color"] = (*tr_c, 1.0 if self.thin_walled else 0.0)
        m["parameters3"] = (self.sheen_roughness, tr_r, tr_ior, self.specular_anisotropy)
        m["clearcoat_color"] = (*tuple(self.clearcoat_color), 0.0)
        m["clearcoat_attenuation"] = (*cc_att, self.clearcoat_thickness)
        m["transmission_absorption"] = (*tuple(self.transmission_absorption_color),
                                        self.transmission_absorption_distance)
        m["thin_film"] = (self.thin_film, self.thin_film_thickness_nanometers, self.thin_film_index_of_refraction, 0.0)
        m["subsurface_color"] = (*sub_c, self.subsurface)
        m["subsurface_radius"] = (*tuple(self.subsurface_radius), self.subsurface_scale)
        m["subsurface_parameters"] = (self.subsurface_anisotropy, 0.0, 0.0, 0.0)
        m["volume_scattering"] = (*vs_c, self.volume_scattering)
        m["volume_parameters"] = (self.volume_scattering_distance, self.volume_anisotropy, 0.0, 0.0)
        return m


# ----------------------------------------------------------------- texture ---
@dataclasses.dataclass
class Texture2D:
    """Texture2D (Scene/Texture.swift:43-67): linear RGBA, row-major."""
    width: int
    height: int
    pixels: np.ndarray  # (height*width, 4) float32
    sampling_mode: int = 0  # 0 nearest, 1 linear


@dataclasses.dataclass
class Environment:
    """Environment (Scene/Environment.swift:4-31)."""
    texture: Optional[Texture2D] = None
    intensity: float = 1.0
    rotation_y: float = 0.0
    max_radiance: float = 16.0


# ------------------------------------------------------------------ bounds ---
@dataclasses.dataclass
class SceneBounds:
    """SceneBounds (Scene/SceneBounds.swift:5-111): an axis-aligned box, empty
    while any minimum exceeds its maximum."""
    minimum: tuple = (math.inf, math.inf, math.inf)
    maximum: tuple = (-math.inf, -math.inf, -math.inf)

    @staticmethod
    def of(a, b) -> "SceneBounds":
        """SceneBounds(minimum:maximum:): the box of two corners in any order."""
        return SceneBounds(tuple(min(float(x), float(y)) for x, y in zip(a, b)),
                           tuple(max(float(x), float(y)) for x, y in zip(a, b)))

    def is_empty(self) -> bool:
        return any(lo > hi for lo, hi in zip(self.minimum, self.maximum))

    def center(self) -> tuple:
        if self.is_empty():
            return (0.0, 0.0, 0.0)
        return tuple((lo + hi) * 0.5 for lo, hi in zip(self.minimum, self.maximum))

    def extent(self) -> tuple:
        if self.is_empty():
            return (0.0, 0.0, 0.0)
        return tuple(hi - lo for lo, hi in zip(self.minimum, self.maximum))

    def corners(self) -> list:
        """The eight corners, x fastest (SceneBounds.swift:69-83)."""
        if self.is_empty():
            return []
        (x0, y0, z0), (x1, y1, z1) = self.minimum, self.maximum
        return [(x, y, z) for z in (z0, z1) for y in (y0, y1) for x in (x0, x1)]

    def including(self, other) -> "SceneBounds":
        """include(_:) for a point (3 numbers) or a non-empty SceneBounds."""
        if isinstance(other, SceneBounds):
            if other.is_empty():
                return self
            return self.including(other.minimum).including(other.maximum)
        return SceneBounds(tuple(min(lo, float(v)) for lo, v in zip(self.minimum, other)),
                           tuple(max(hi, float(v)) for hi, v in zip(self.maximum, other)))

    def transformed(self, transform: "Transform") -> "SceneBounds":
        """transformed(by:) (SceneBounds.swift:100-110): the box of the transformed corners."""
        if self.is_empty():
            return SceneBounds()
        pts = transform.transform_points(np.asarray(self.corners(), f32))
        out = SceneBounds()
        for p in pts:
            out = out.including(tuple(float(v) for v in p))
        return out


# ------------------------------------------------------------------ camera ---
@dataclasses.dataclass
class Camera:
    """Camera (Scene/Camera.swift:44-243)."""
    origin: Sequence[float]
    target: Sequence[float]
    up: Sequence[float] = (0.0, 1.0, 0.0)
    vertical_field_of_view_degrees: float = 45.0
    orthographic_scale: Optional[float] = None  # None: perspective
    focus_distance: float = 1.0
    aperture_radius: float = 0.0

    def gpu_camera(self, width: int, height: int) -> abi.Camera:
        """Camera.gpuCamera (Camera.swift:167-200) with cameraBasis (:202-218).

        Scalar float32 arithmetic, each operation rounded to float32 in the
        order of the reference's simd code (dot and length as ((x + y) + z),
        cross products as a*b - c*d without fusion); a request-rate path of
        the render server, so no per-call array allocation."""
        o = tuple(f32(c) for c in self.origin)
        t = tuple(f32(c) for c in self.target)
        vd = (t[0] - o[0], t[1] - o[1], t[2] - o[2])
        forward = _normalize3(vd) if float(_dot3(vd, vd)) > 1e-8 else (f32(0), f32(0), f32(-1))
        u = tuple(f32(c) for c in self.up)
        up = _normalize3(u) if float(_dot3(u, u)) > 1e-8 else (f32(0), f32(1), f32(0))
        helper = up if abs(float(_dot3(forward, up))) < 0.999 else (f32(1), f32(0), f32(0))
        right = _normalize3(_cross3(forward, helper))
        true_up = _cross3(right, forward)
        aspect = f32(width) / f32(height)
        if self.orthographic_scale is None:
            theta = f32(self.vertical_field_of_view_degrees) * f32(math.pi) / f32(180)
            vh = f32(2) * f32(math.tan(theta / f32(2)))
            flag = 0.0
        else:
            vh = f32(max(self.orthographic_scale, 0.0001))
            flag = 1.0
        vw = f32(aspect * vh)
        horizontal = tuple(vw * c for c in right)
        vertical = tuple(vh * c for c in true_up)
        pc = tuple(o[i] + forward[i] for i in range(3)) if self.orthographic_scale is None else o
        half = f32(0.5)
        lower_left = tuple((pc[i] - horizontal[i] * half) - vertical[i] * half for i in range(3))
        cam = abi.Camera()
        cam.origin = abi.Float4(float(o[0]), float(o[1]), float(o[2]), flag)
        cam.lower_left = abi.Float4(*(float(c) for c in lower_left), 0.0)
        cam.horizontal = abi.Float4(*(float(c) for c in horizontal), 0.0)
        cam.vertical = abi.Float4(*(float(c) for c in vertical), 0.0)
        cam.lens = abi.Float4(max(self.aperture_radius, 0.0), max(self.focus_distance, 0.0001), 0.0, 0.0)
        return cam

    def view_direction(self) -> tuple:
        """Camera.viewDirection (Camera.swift:80-87): the normalised origin -> target
        vector, (0, 0, -1) when the two points coincide."""
        o = tuple(f32(c) for c in self.origin)
        vd = tuple(f32(c) - o[i] for i, c in enumerate(self.target))
        return _normalize3(vd) if float(_dot3(vd, vd)) > 1e-8 else (f32(0), f32(0), f32(-1))

    def focused(self, point: Sequence[float], aperture_radius: float) -> "Camera":
        """Camera.focused(on:apertureRadius:) (Camera.swift:89-101): a copy whose focal
        plane passes through `point` (its distance along the view direction, at
        least 0.0001) with the given aperture radius (at least 0)."""
        o = tuple(f32(c) for c in self.origin)
        rel = tuple(f32(c) - o[i] for i, c in enumerate(point))
        distance = max(float(_dot3(rel, self.view_direction())), 0.0001)
        return dataclasses.replace(self, focus_distance=distance, aperture_radius=max(float(aperture_radius), 0.0))

    @staticmethod
    def framing(bounds: SceneBounds, aspect_ratio: float, view_direction=(0.0, -0.25, -1.0), up=(0.0, 1.0, 0.0),
                padding: float = 1.15, center_offset=(0.0, 0.0), target_offset=(0.0, 0.0, 0.0),
                orthographic: bool = False, vertical_field_of_view_degrees: float = 45.0,
                aperture_radius: float = 0.0) -> "Camera":
        """Camera.framing (Camera.swift:103-165): a camera looking along
        `view_direction` that fits the padded corners of `bounds`, perspective
        (the field of view clamped to 1-175 degrees) or orthographic (vertical
        scale from the fitted extents).  `center_offset` moves the bounds'
        centre on the image in fitted-frame units (+x right, +y up)."""
        def basis(view, upv):
            v = tuple(float(c) for c in view)
            fwd = _normalize3(v) if _dot3(v, v) > 1e-8 else (0.0, 0.0, -1.0)
            u = tuple(float(c) for c in upv)
            u = _normalize3(u) if _dot3(u, u) > 1e-8 else (0.0, 1.0, 0.0)
            helper = u if abs(_dot3(fwd, u)) < 0.999 else (1.0, 0.0, 0.0)
            right = _normalize3(_cross3(fwd, helper))
            return fwd, right, _cross3(right, fwd)

        def extents(corners, center, b):
            fwd, right, tup = b
            hw = hh = 0.0
            zs = []
            for c in corners:
                rel = tuple(c[i] - center[i] for i in range(3))
                hw = max(hw, abs(_dot3(rel, right)))
                hh = max(hh, abs(_dot3(rel, tup)))
                zs.append(_dot3(rel, fwd))
            return max(hw, 0.0001), max(hh, 0.0001), max(max(zs) - min(zs), 0.0001)

        fwd, right, tup = b = basis(view_direction, up)
        bc = bounds.center()
        center = tuple(bc[i] + float(target_offset[i]) for i in range(3))
        pad = max(float(padding), 0.0001)
        corners = [tuple(center[i] + (c[i] - bc[i]) * pad for i in range(3)) for c in bounds.corners()]
        aspect = max(float(aspect_ratio), 0.0001)
        hw, hh, _ = extents(corners, center, b)
        shift = tuple(right[i] * (hw * float(center_offset[0])) + tup[i] * (hh * float(center_offset[1]))
                      for i in range(3))
        target = tuple(center[i] - shift[i] for i in range(3))
        if not orthographic:
            fov = min(max(float(vertical_field_of_view_degrees), 1.0), 175.0)
            tan_y = math.tan(fov * math.pi / 360.0)
            tan_x = tan_y * aspect
            distance = 0.0001
            for c in corners:
                rel = tuple(c[i] - target[i] for i in range(3))
                x, y, z = _dot3(rel, right), _dot3(rel, tup), _dot3(rel, fwd)
                distance = max(distance, abs(x) / max(tan_x, 0.0001) - z, abs(y) / max(tan_y, 0.0001) - z)
            origin = tuple(target[i] - fwd[i] * distance for i in range(3))
            return Camera(origin, target, up=tup, vertical_field_of_view_degrees=fov, focus_distance=distance,
                          aperture_radius=max(float(aperture_radius), 0.0))
        thw, thh, depth = extents(corners, target, b)
        scale = max(thh, thw / aspect) * 2.0
        distance = max(depth * 0.5 + max(thw, thh), 0.0001)
        origin = tuple(target[i] - fwd[i] * distance for i in range(3))
        return Camera(origin, target, up=tup, orthographic_scale=max(scale, 0.0001), focus_distance=distance,
                      aperture_radius=max(float(aperture_radius), 0.0))


# ------------------------------------------------------------ render scene ---
@dataclasses.dataclass
class MeshInstance:
    mesh: Mesh
    material: int
    transform: Transform = dataclasses.field(default_factory=Transform.identity)


@dataclasses.dataclass
class RenderScene:
    """RenderScene (Scene/RenderScene.swift:73-130): materials, mesh instances,
    camera and environment."""
    camera: Camera = dataclasses.field(default_factory=lambda: Camera((0, 0, 3), (0, 0, 0)))
    environment: Environment = dataclasses.field(default_factory=Environment)
    materials: List[Material] = dataclasses.field(default_factory=list)
    mesh_instances: List[MeshInstance] = dataclasses.field(default_factory=list)
    # Pre-built triangle arrays appended after the instances (a bulk path for
    # large generated scenes; same layout as materialised instances).
    extra_triangles: List[np.ndarray] = dataclasses.field(default_factory=list)
    # Sparse distance volumes (library.SparseVolume), bound after the meshes.
    sparse_volumes: List[object] = dataclasses.field(default_factory=list)

    def add_material(self, m: Material) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add(self, mesh: Mesh, material: int, transform: Optional[Transform] = None) -> None:
        self.mesh_instances.append(MeshInstance(mesh, material, transform or Transform.identity()))

    def world_bounds(self) -> Optional[SceneBounds]:
        """RenderScene.worldBounds (SceneBounds.swift:136-170): the mesh
        instances' transformed vertex bounds and the sparse volumes' bounds;
        None for an empty scene."""
        out = SceneBounds()
        for inst in self.mesh_instances:
            v = np.asarray(inst.mesh.vertices, f32)
            if len(v) == 0:
                continue
            local = SceneBounds.of(v.min(axis=0), v.max(axis=0))
            out = out.including(local.transformed(inst.transform))
        for vol in self.sparse_volumes:
            lo, hi = getattr(vol, "bounds_min", None), getattr(vol, "bounds_max", None)
            if lo is not None and hi is not None:
                out = out.including(SceneBounds.of(lo, hi))
        return None if out.is_empty() else out

    def add_quad_light(self, light: "QuadLight") -> int:
        """RenderScene.addQuadLight (RenderScene.swift:307-321): the light's
        emissive material and its quad; returns the material index.  Scenes
        get no lights by default."""
        material = self.add_material(light.material())
        self.add(Mesh.quad(light.a, light.b, light.c, light.d), material)
        return material


@dataclasses.dataclass
class QuadLight:
    """QuadLight (Scene/QuadLight.swift:5-50): a rectangular area light from
    four corners, emitting `color` x `intensity`."""
    a: Sequence[float]
    b: Sequence[float]
    c: Sequence[float]
    d: Sequence[float]
    color: Sequence[float] = (1.0, 1.0, 1.0)
    intensity: float = 1.0

    def material(self) -> Material:
        """The light's material (QuadLight.swift:41-50)."""
        return Material(base_color=tuple(self.color), emission=tuple(self.color), emission_strength=self.intensity,
                        roughness=0.4, metallic=0.0, specular=0.0)


@dataclasses.dataclass
class AccelerationBuild:
    """The POD arrays of AccelerationBuild (Acceleration/AccelerationBuild.swift:4-48)
    that the C ABI receives, plus the environment settings."""
    triangles: np.ndarray
    materials: np.ndarray
    nodes: np.ndarray
    primitive_indices: np.ndarray
    texture_descriptors: np.ndarray
    texture_pixels: np.ndarray
    lights: np.ndarray
    environment_samples: np.ndarray
    environment_texture_index_plus_one: int
    environment_intensity: float
    environment_rotation_y: float
    environment_max_radiance: float
    volumes: Optional[np.ndarray] = None
    volume_bricks: Optional[np.ndarray] = None
    volume_brick_samples: Optional[np.ndarray] = None
    volume_brick_grids: Optional[np.ndarray] = None
    volume_brick_grid_indices: Optional[np.ndarray] = None

    def as_struct(self) -> abi.Scene:
        """dk_scene view over the arrays (the arrays must outlive the struct)."""
        s = abi.Scene()

        def ptr(a):
            return a.ctypes.data if a is not None and len(a) else None

        s.triangles, s.triangle_count = ptr(self.triangles), len(self.triangles)
        s.materials, s.material_count = ptr(self.materials), len(self.materials)
        s.nodes, s.node_count = ptr(self.nodes), len(self.nodes)
        s.primitive_indices, s.primitive_index_count = ptr(self.primitive_indices), len(self.primitive_indices)
        s.texture_descriptors, s.texture_descriptor_count = ptr(self.texture_descriptors), len(self.texture_descriptors)
        s.texture_pixels, s.texture_pixel_count = ptr(self.texture_pixels), len(self.texture_pixels)
        s.lights, s.light_count = ptr(self.lights), len(self.lights)
        s.environment_samples, s.environment_sample_count = (ptr(self.environment_samples),
                                                             len(self.environment_samples))
        s.environment_texture_index_plus_one = self.environment_texture_index_plus_one
        s.environment_intensity = self.environment_intensity
        s.environment_rotation_y = self.environment_rotation_y
        s.environment_max_radiance = self.environment_max_radiance
        for name in ("volumes", "volume_bricks", "volume_brick_samples", "volume_brick_grids",
                     "volume_brick_grid_indices"):
            a = getattr(self, name)
            setattr(s, name, ptr(a))
            setattr(s, name.rstrip("s") + "_count" if name != "volume_brick_grid_indices" else
                    "volume_brick_grid_index_count", 0 if a is None else len(a))
        return s


def compile_scene(scene: RenderScene, build_bvh: bool = True, host_builders=None) -> AccelerationBuild:
    """LinearTriangleAccelerationBackend.build (AccelerationBackend.swift:7-68).

    The BVH, light list and environment table come from the GB300 library
    (`dk_build_bvh`, `dk_build_lights`, `dk_build_environment_samples`);
    `host_builders` — any object with the same three functions — replaces
    them (the test oracle passes its restatement of the Swift builders)."""
    from . import library  # the scene-compile helpers live in the GB300 library
    builders = host_builders or library

    # InstanceAccelerationBuilder.build + materializedTriangles
    # (InstanceAcceleration.swift:23-128): local triangles with identity
    # transform, then the instance transform, materialID and objectID.
    parts = []
    cache = {}
    for object_id, inst in enumerate(scene.mesh_instances):
        if inst.material >= len(scene.materials):
            raise ValueError("Invalid render scene: Mesh references an unknown material.")
        key = id(inst.mesh)
        if key not in cache:
            cache[key] = inst.mesh.gpu_triangles(0, Transform.identity(), 0)
        local = cache[key]
        tris = local.copy()
        t = inst.transform
        for name in ("v0", "v1", "v2"):
            if not t.is_identity():
                tris[name][:, :3] = t.transform_points(local[name][:, :3])
        for name in ("n0", "n1", "n2", "tangent", "bitangent"):
            tris[name][:, :3] = t.transform_normals(local[name][:, :3])
        tris["material_id"] = inst.material
        tris["object_id"] = object_id
        tris["padding2"] = 0
        parts.append(tris)
    parts.extend(scene.extra_triangles)
    triangles = np.concatenate(parts) if parts else np.zeros(0, abi.TRIANGLE_DTYPE)
    triangles = np.ascontiguousarray(triangles)

    # gpuMaterialsAndTextures (MaterialGPUEncoding.swift:5-50)
    descriptors, pixels = [], []
    pixel_count = 0

    def append(tex: Optional[Texture2D]) -> Optional[int]:
        nonlocal pixel_count
        if tex is None or tex.width <= 0 or tex.height <= 0:
            return None
        n = tex.width * tex.height
        if len(tex.pixels) < n:
            return None
        d = np.zeros((), abi.TEXTURE_DESCRIPTOR_DTYPE)
        d["metadata"] = (pixel_count, tex.width, tex.height, tex.sampling_mode)
        descriptors.append(d)
        pixels.append(np.asarray(tex.pixels[:n], f32).reshape(n, 4))
        pixel_count += n
        return len(descriptors) - 1

    mats = []
    for m in scene.materials:
        bi = append(m.base_color_texture)
        ni = append(m.normal_map)
        mats.append(m.gpu_material(bi, ni))
    env_index = append(scene.environment.texture)
    env_plus_one = 0 if env_index is None else env_index + 1
    materials = np.array(mats, dtype=abi.MATERIAL_DTYPE) if mats else np.zeros(0, abi.MATERIAL_DTYPE)
    texture_descriptors = (np.array(descriptors, abi.TEXTURE_DESCRIPTOR_DTYPE) if descriptors
                           else np.zeros(0, abi.TEXTURE_DESCRIPTOR_DTYPE))
    texture_pixels = np.concatenate(pixels) if pixels else np.zeros((0, 4), f32)

    lights = builders.build_lights(triangles, materials)
    if build_bvh:
        nodes, prim = builders.build_bvh(triangles, 4)
    else:
        nodes, prim = np.zeros(0, abi.NODE_DTYPE), np.zeros(0, np.uint32)
    env = scene.environment
    if env.texture is not None:
        env_samples = builders.build_environment_samples(env.texture, env.intensity, env.max_radiance)
    else:
        env_samples = np.zeros(0, abi.ENVIRONMENT_SAMPLE_DTYPE)
    vols = {}
    if scene.sparse_volumes:
        if len(scene.sparse_volumes) > 1:
            raise ValueError("Invalid render scene: one sparse distance volume per scene is supported.")
        sv = scene.sparse_volumes[0]
        vols = dict(volumes=sv.volumes, volume_bricks=sv.bricks, volume_brick_samples=sv.samples,
                    volume_brick_grids=sv.grids, volume_brick_grid_indices=sv.grid_indices)
    return AccelerationBuild(
        **vols,
        triangles=triangles, materials=materials, nodes=nodes, primitive_indices=prim,
        texture_descriptors=texture_descriptors, texture_pixels=np.ascontiguousarray(texture_pixels, f32),
        lights=lights, environment_samples=env_samples, environment_texture_index_plus_one=env_plus_one,
        environment_intensity=float(env.intensity), environment_rotation_y=float(env.rotation_y),
        environment_max_radiance=float(env.max_radiance))
