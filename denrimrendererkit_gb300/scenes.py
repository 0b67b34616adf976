"""Seeded synthetic scenes: the benchmark configurations and the reference's
own test scenes.

* `cornell_small()`  — the small plain-method configuration: a Cornell-style box
  of 5 Lambert quads (albedo 0.73, red/green side walls), a 0.25 x 0.25
  emissive ceiling quad (radiance 17, 12, 4) and a subdivision-3 icosphere
  (1,280 triangles, r = 0.3) with the `matte.clay` preset
  (Scene/BuiltInMaterialLibrary.swift:62-67); pinhole camera, fov 40 degrees,
  320x180, 16 spp, 8 bounces, frame seed 1.
* `spheres_large()`  — the large plain-method configuration: 64 seeded
  noise-displaced subdivision-5 icospheres (20,480 triangles each), a 2-tri
  ground plane, 16 emissive triangles, a 2048x1024 HDRI with log-normal texel
  luminance (mu 0, sigma 1.5) and a 2-degree sun of 1e4x peak; materials drawn
  uniformly from diffuse / GGX metal (roughness U[0.05, 0.8]) / dielectric
  (IOR 1.5) / clearcoat; 1920x1080, 64 spp, 12 bounces, maxRadiance and the
  sample clamp both off so the sun is not clipped.
* `cornell_box_reference()`, `parity_quad_scene()`,
  `reused_mesh_instance_scene()` — RenderScene.cornellBox
  (Scene/RenderScene.swift:324-380) and the scenes of
  Tests/DenrimRendererKitTests/HardwareTraversalParityTests.swift:168-224.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .renderer import RenderQuality, RenderSettings
from .scene import Camera, Environment, Material, Mesh, RenderScene, Texture2D, Transform, icosphere

f32 = np.float32


@dataclasses.dataclass
class Workload:
    name: str
    scene: RenderScene
    settings: RenderSettings
    samples: int


MATTE_CLAY = dict(base_color=(0.78, 0.62, 0.48), roughness=0.82, specular=0.25)


def cornell_small(width: int = 320, height: int = 180, samples: int = 16) -> Workload:
    scene = RenderScene(camera=Camera((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), vertical_field_of_view_degrees=40.0))
    grey = scene.add_material(Material(base_color=(0.73, 0.73, 0.73), specular=0.0))
    red = scene.add_material(Material(base_color=(0.65, 0.05, 0.05), specular=0.0))
    green = scene.add_material(Material(base_color=(0.12, 0.45, 0.15), specular=0.0))
    light = scene.add_material(Material(base_color=(1.0, 1.0, 1.0), emission=(17.0, 12.0, 4.0), emission_strength=1.0))
    clay = scene.add_material(Material(**MATTE_CLAY))
    scene.add(Mesh.quad((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1)), grey)      # floor
    scene.add(Mesh.quad((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)), grey)      # ceiling
    scene.add(Mesh.quad((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)), grey)    # back
    scene.add(Mesh.quad((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1)), red)     # left
    scene.add(Mesh.quad((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)), green)       # right
    scene.add(Mesh.quad((-0.125, 1.99, -0.125), (0.125, 1.99, -0.125), (0.125, 1.99, 0.125),
                        (-0.125, 1.99, 0.125)), light)
    scene.add(icosphere(3, 0.3), clay, Transform.translation((0.0, 0.3, 0.0)))
    settings = RenderSettings(width=width, height=height, max_bounces=8, quality=RenderQuality.FINAL,
                              frame_seed=1)
    return Workload("cornell-small-320x180-16spp", scene, settings, samples)


def cornell_variant(seed: int, width: int = 256, height: int = 256, samples: int = 4) -> Workload:
    """A reseeded variant of the small configuration, for denoiser training
    pairs: wall colours, the ceiling light's size and power, a sphere with a
    material drawn from the preset library (position, radius) and a box with a
    random diffuse colour, size and rotation are drawn from `seed`."""
    from .presets import PRESETS
    rng = np.random.default_rng(seed)
    cam = Camera((float(rng.uniform(-0.15, 0.15)), float(rng.uniform(0.9, 1.1)), float(rng.uniform(3.2, 3.6))),
                 (0.0, 1.0, 0.0), vertical_field_of_view_degrees=float(rng.uniform(36.0, 44.0)))
    scene = RenderScene(camera=cam)

    def col(lo, hi):
        return tuple(float(v) for v in rng.uniform(lo, hi, 3))

    grey = scene.add_material(Material(base_color=col(0.55, 0.8), specular=0.0))
    left = scene.add_material(Material(base_color=col(0.05, 0.8), specular=0.0))
    right = scene.add_material(Material(base_color=col(0.05, 0.8), specular=0.0))
    power = float(rng.uniform(0.6, 1.4))
    light = scene.add_material(Material(base_color=(1.0, 1.0, 1.0), emission=(17.0 * power, 12.0 * power, 4.0 * power),
                                         emission_strength=1.0))
    names = sorted(PRESETS)
    sphere = scene.add_material(PRESETS[names[int(rng.integers(0, len(names)))]])
    box = scene.add_material(Material(base_color=col(0.1, 0.9), roughness=float(rng.uniform(0.3, 0.9)),
                                      specular=float(rng.uniform(0.0, 0.5))))
    scene.add(Mesh.quad((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1)), grey)
    scene.add(Mesh.quad((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)), grey)
    scene.add(Mesh.quad((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)), grey)
    scene.add(Mesh.quad((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1)), left)
    scene.add(Mesh.quad((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)), right)
    hl = float(rng.uniform(0.1, 0.3))
    scene.add(Mesh.quad((-hl, 1.99, -hl), (hl, 1.99, -hl), (hl, 1.99, hl), (-hl, 1.99, hl)), light)
    r = float(rng.uniform(0.2, 0.4))
    scene.add(icosphere(3, r), sphere, Transform.translation((float(rng.uniform(-0.5, 0.1)), r,
                                                             float(rng.uniform(-0.4, 0.4)))))
    bh = float(rng.uniform(0.3, 1.1))
    bw = float(rng.uniform(0.2, 0.35))
    scene.add(Mesh.box((-bw, 0.0, -bw), (bw, bh, bw)), box,
              Transform.translation((float(rng.uniform(0.3, 0.6)), 0.0, float(rng.uniform(-0.5, 0.2))))
              * Transform.rotation_y(float(rng.uniform(0.0, 1.5))))
    settings = RenderSettings(width=width, height=height, max_bounces=8, quality=RenderQuality.FINAL,
                              frame_seed=int(rng.integers(1, 2 ** 31)))
    return Workload(f"cornell-variant-{seed}-{width}x{height}-{samples}spp", scene, settings, samples)


def _displaced_icosphere(rng: np.random.Generator, subdivisions: int, radius: float, amplitude: float) -> Mesh:
    base = icosphere(subdivisions, 1.0)
    v = base.vertices.astype(np.float64)
    dirs = rng.normal(size=(4, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    freq = rng.uniform(2.0, 7.0, size=4)
    phase = rng.uniform(0.0, 2 * math.pi, size=4)
    noise = np.sin((v @ dirs.T) * freq + phase).sum(axis=1) / 4.0
    pos = v * (radius * (1.0 + amplitude * noise))[:, None]
    tri = base.indices.reshape(-1, 3).astype(np.int64)
    fn = np.cross(pos[tri[:, 1]] - pos[tri[:, 0]], pos[tri[:, 2]] - pos[tri[:, 0]])
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, tri[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    return Mesh(pos.astype(f32), base.indices, normals=vn.astype(f32))


def synthetic_hdri(width: int = 2048, height: int = 1024, seed: int = 2, sigma: float = 1.5,
                   sun_peak: float = 1.0e4, sun_radius_deg: float = 1.0,
                   sun_dir=(0.45, 0.55, -0.70)) -> Texture2D:
    """Equirectangular HDRI with log-normal texel luminance and a sun disc of
    `sun_peak` times the log-normal level, in the reference's mapping
    (u = atan2(z, x) / 2pi + 0.5, v = acos(y) / pi; PathTrace.metal:3785-3787)."""
    rng = np.random.default_rng(seed)
    lum = np.exp(rng.normal(0.0, sigma, size=(height, width)))
    tint = np.stack([np.full_like(lum, 1.0), np.full_like(lum, 0.95), np.full_like(lum, 1.1)], axis=-1)
    y = (np.arange(height) + 0.5) / height
    x = (np.arange(width) + 0.5) / width
    theta = y[:, None] * math.pi
    phi = (x[None, :] - 0.5) * 2 * math.pi
    d = np.stack([np.cos(phi) * np.sin(theta), np.cos(theta) * np.ones_like(phi), np.sin(phi) * np.sin(theta)], -1)
    s = np.asarray(sun_dir, np.float64)
    s /= np.linalg.norm(s)
    cosang = d @ s
    sun = cosang >= math.cos(math.radians(sun_radius_deg))
    lum = np.where(sun, lum * sun_peak, lum)
    rgb = lum[..., None] * tint
    px = np.concatenate([rgb, np.ones((height, width, 1))], axis=-1).astype(f32).reshape(-1, 4)
    return Texture2D(width, height, px, sampling_mode=1)


def spheres_large(width: int = 1920, height: int = 1080, samples: int = 64, seed: int = 7,
                  subdivisions: int = 5, hdri_size=(2048, 1024)) -> Workload:
    rng = np.random.default_rng(seed)
    env = Environment(texture=synthetic_hdri(*hdri_size), intensity=1.0, rotation_y=0.0, max_radiance=0.0)
    scene = RenderScene(camera=Camera((0.0, 5.5, 10.5), (0.0, 0.4, 0.0), vertical_field_of_view_degrees=40.0),
                        environment=env)
    ground = scene.add_material(Material(base_color=(0.55, 0.55, 0.52), roughness=0.9, specular=0.2))
    scene.add(Mesh.quad((-12, 0, 12), (12, 0, 12), (12, 0, -12), (-12, 0, -12)), ground)
    families = ("diffuse", "metal", "dielectric", "clearcoat")
    for i in range(64):
        fam = families[int(rng.integers(0, 4))]
        col = tuple(float(c) for c in rng.uniform(0.2, 0.95, size=3))
        if fam == "diffuse":
            m = Material(base_color=col, roughness=0.8, specular=0.0)
        elif fam == "metal":
            m = Material(base_color=col, metallic=1.0, roughness=float(rng.uniform(0.05, 0.8)))
        elif fam == "dielectric":
            m = Material(base_color=(1.0, 1.0, 1.0), roughness=0.0, transmission=1.0, index_of_refraction=1.5)
        else:
            m = Material(base_color=col, roughness=0.5, clearcoat=1.0, clearcoat_roughness=0.05)
        mi = scene.add_material(m)
        gx, gz = i % 8, i // 8
        center = (-4.2 + 1.2 * gx, 0.5, -4.2 + 1.2 * gz)
        mesh = _displaced_icosphere(rng, subdivisions, 0.45, 0.08)
        scene.add(mesh, mi, Transform.translation(center))
    warm = scene.add_material(Material(base_color=(1, 1, 1), emission=(1.0, 0.8, 0.6), emission_strength=40.0))
    cool = scene.add_material(Material(base_color=(1, 1, 1), emission=(0.6, 0.75, 1.0), emission_strength=40.0))
    for k in range(8):
        cx, cz = -3.5 + k, -2.0 + 1.5 * (k % 3)
        h = 0.15
        scene.add(Mesh.quad((cx - h, 3.5, cz - h), (cx + h, 3.5, cz - h), (cx + h, 3.5, cz + h), (cx - h, 3.5, cz + h)),
                  warm if k % 2 == 0 else cool)
    settings = RenderSettings(width=width, height=height, max_bounces=12, quality=RenderQuality.FINAL,
                              sample_radiance_clamp=0.0, frame_seed=1)
    return Workload(f"spheres-large-{width}x{height}-{samples}spp", scene, settings, samples)


def sdf_spheres(width: int = 1024, height: int = 1024, samples: int = 16, resolution: int = 768, seed: int = 5,
                narrow_band: float = 0.012, fp16: bool = True) -> Workload:
    """The sparse-SDF configuration: 32 seeded spheres (radii U[0.03, 0.15],
    centres in [-0.85, 0.85]^3) joined by a polynomial smooth union (k = 0.05),
    baked into a `resolution`^3 virtual grid over [-1, 1]^3 with 8^3-sample
    bricks; a narrow band of 0.012 keeps 3.0% of the 96^3 bricks at 768^3.
    Distances stored as FP16 (`fp16`; False keeps FP32).  Spheres alternate a
    diffuse and a GGX metal material; lit by the default sky.  1024x1024,
    16 spp."""
    from .library import SparseVolume
    rng = np.random.default_rng(seed)
    scene = RenderScene(camera=Camera((0.0, 0.9, 3.1), (0.0, 0.0, 0.0), vertical_field_of_view_degrees=40.0))
    diffuse = scene.add_material(Material(base_color=(0.7, 0.55, 0.4), roughness=0.8, specular=0.0))
    metal = scene.add_material(Material(base_color=(0.9, 0.9, 0.95), metallic=1.0, roughness=0.25))
    spheres = [dict(center=rng.uniform(-0.85, 0.85, 3), radius=float(rng.uniform(0.03, 0.15)),
                    material=(diffuse if i % 2 == 0 else metal), smooth_union_radius=0.05) for i in range(32)]
    vol = SparseVolume(spheres, (resolution,) * 3, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), (8, 8, 8), narrow_band,
                       volume_material=diffuse, object_id=0, primitive_id=0, fp16_distances=fp16)
    scene.sparse_volumes.append(vol)
    settings = RenderSettings(width=width, height=height, max_bounces=8, quality=RenderQuality.FINAL, frame_seed=1)
    return Workload(f"sdf-spheres-{resolution}^3-{width}x{height}-{samples}spp-{'fp16' if fp16 else 'fp32'}", scene,
                    settings, samples)


def _checker(width: int, height: int, a, b, cells: int = 8) -> Texture2D:
    y, x = np.mgrid[0:height, 0:width]
    mask = ((x * cells // width + y * cells // height) % 2).astype(bool)
    rgb = np.where(mask[..., None], np.asarray(a, np.float64), np.asarray(b, np.float64))
    px = np.concatenate([rgb, np.ones((height, width, 1))], axis=-1).astype(f32).reshape(-1, 4)
    return Texture2D(width, height, px, sampling_mode=1)


def _bump_normal_map(width: int, height: int, seed: int) -> Texture2D:
    rng = np.random.default_rng(seed)
    n = rng.normal(0.0, 0.25, size=(height, width, 2))
    xyz = np.concatenate([n, np.ones((height, width, 1))], axis=-1)
    xyz /= np.linalg.norm(xyz, axis=-1, keepdims=True)
    enc = xyz * 0.5 + 0.5
    px = np.concatenate([enc, np.ones((height, width, 1))], axis=-1).astype(f32).reshape(-1, 4)
    return Texture2D(width, height, px, sampling_mode=0)


def material_zoo(width: int = 96, height: int = 64, samples: int = 8, seed: int = 11) -> Workload:
    """Feature-coverage scene: one subdivision-2 icosphere per material feature
    of the layered BSDF (Scene/Material.swift:16-219) — thin film, sheen,
    anisotropic GGX metal, clearcoat with thickness and attenuation, random-walk
    subsurface, rough and thin-walled transmission with Beer absorption, a
    scattering interior medium, a cut-out (opacity 0.5), a checker base-colour
    texture and a normal map — on a textured ground under a rotated HDRI with
    maxRadiance clipping, two emissive quads, and the per-sample radiance clamp
    at its `final` default."""
    rng = np.random.default_rng(seed)
    env = Environment(texture=synthetic_hdri(256, 128, seed=seed, sun_peak=200.0, sun_radius_deg=4.0),
                      intensity=0.8, rotation_y=0.7, max_radiance=24.0)
    scene = RenderScene(camera=Camera((0.0, 2.4, 6.2), (0.0, 0.45, 0.0), vertical_field_of_view_degrees=38.0),
                        environment=env)
    ground = scene.add_material(Material(base_color=(0.7, 0.7, 0.7), roughness=0.7, specular=0.5,
                                         base_color_texture=_checker(64, 64, (0.8, 0.78, 0.7), (0.25, 0.27, 0.3))))
    scene.add(Mesh.quad((-6, 0, 6), (6, 0, 6), (6, 0, -6), (-6, 0, -6)), ground)
    presets = [
        Material(base_color=(0.3, 0.35, 0.4), metallic=1.0, roughness=0.25, thin_film=1.0,
                 thin_film_thickness_nanometers=380.0),
        Material(base_color=(0.35, 0.08, 0.12), roughness=0.9, specular=0.3, sheen=1.0, sheen_color=(1.0, 0.9, 0.9),
                 sheen_roughness=0.4),
        Material(base_color=(0.95, 0.7, 0.35), metallic=1.0, roughness=0.35, specular_anisotropy=0.8),
        Material(base_color=(0.6, 0.05, 0.05), roughness=0.45, clearcoat=1.0, clearcoat_roughness=0.08,
                 clearcoat_thickness=0.6, clearcoat_attenuation_color=(0.9, 0.7, 0.3)),
        Material(base_color=(0.9, 0.75, 0.65), roughness=0.5, subsurface=0.9, subsurface_color=(0.95, 0.6, 0.45),
                 subsurface_radius=(0.5, 0.25, 0.12), subsurface_scale=0.3, subsurface_anisotropy=0.2),
        Material(base_color=(1.0, 1.0, 1.0), roughness=0.15, transmission=1.0, index_of_refraction=1.45,
                 transmission_roughness=0.2, transmission_absorption_color=(0.4, 0.8, 0.6),
                 transmission_absorption_distance=0.5),
        Material(base_color=(1.0, 1.0, 1.0), roughness=0.0, transmission=1.0, thin_walled=True,
                 transmission_color=(0.8, 0.9, 1.0)),
        Material(base_color=(0.95, 0.95, 0.92), roughness=0.2, transmission=1.0, index_of_refraction=1.35,
                 volume_scattering=1.0, volume_scattering_color=(0.9, 0.9, 0.85), volume_scattering_distance=0.2,
                 volume_anisotropy=0.3),
        Material(base_color=(0.2, 0.6, 0.3), roughness=0.6, opacity=0.5),
        Material(base_color=(1.0, 1.0, 1.0), roughness=0.4, specular=0.6,
                 base_color_texture=_checker(32, 32, (0.9, 0.3, 0.1), (0.1, 0.3, 0.9), cells=4)),
        Material(base_color=(0.75, 0.75, 0.8), metallic=0.5, roughness=0.3, normal_map=_bump_normal_map(32, 32, seed)),
        Material(base_color=(0.5, 0.5, 0.5), roughness=0.3, specular=1.0, metallic=0.0),
    ]
    for i, m in enumerate(presets):
        mi = scene.add_material(m)
        gx, gz = i % 4, i // 4
        center = (-2.1 + 1.4 * gx + float(rng.uniform(-0.05, 0.05)), 0.5, -1.4 + 1.4 * gz)
        scene.add(icosphere(2, 0.5), mi, Transform.translation(center) * Transform.rotation_y(0.3 * i))
    warm = scene.add_material(Material(base_color=(1, 1, 1), emission=(1.0, 0.85, 0.6), emission_strength=12.0))
    scene.add(Mesh.quad((-0.5, 3.2, -0.3), (0.5, 3.2, -0.3), (0.5, 3.2, 0.3), (-0.5, 3.2, 0.3)), warm)
    scene.add(Mesh.quad((2.8, 0.2, 1.5), (2.8, 0.2, 0.5), (2.8, 1.4, 0.5), (2.8, 1.4, 1.5)), warm)
    settings = RenderSettings(width=width, height=height, max_bounces=8, quality=RenderQuality.FINAL, frame_seed=1)
    return Workload(f"material-zoo-{width}x{height}-{samples}spp", scene, settings, samples)


def material_preview(hdri=None, subdivisions: int = 4) -> RenderScene:
    """The material-preview scene of the serving workload: a subdivision-4
    icosphere (5,120 triangles, r = 0.5) resting on a 2-triangle ground plane
    under the large configuration's HDRI.  Material 0 is the ground, material 1
    the sphere (the one a job replaces)."""
    env = Environment(texture=hdri if hdri is not None else synthetic_hdri(), intensity=1.0, rotation_y=0.0,
                      max_radiance=0.0)
    scene = RenderScene(camera=Camera((0.0, 0.75, 2.6), (0.0, 0.45, 0.0), vertical_field_of_view_degrees=35.0),
                        environment=env)
    ground = scene.add_material(Material(base_color=(0.5, 0.5, 0.48), roughness=0.85, specular=0.2))
    sphere = scene.add_material(Material(**MATTE_CLAY))
    scene.add(Mesh.quad((-4, 0, 4), (4, 0, 4), (4, 0, -4), (-4, 0, -4)), ground)
    scene.add(icosphere(subdivisions, 0.5), sphere, Transform.translation((0.0, 0.5, 0.0)))
    return scene


@dataclasses.dataclass
class PreviewJob:
    arrival_s: float
    width: int
    height: int
    samples: int
    family: str
    preset: str


def serving_jobs(count: int = 4096, rate_per_s: float = 200.0, seed: int = 3):
    """The serving workload: `count` material-preview jobs with Poisson
    arrivals (rate 200/s), square resolutions {96: 50%, 256: 30%, 512: 15%,
    1024: 5%}, samples uniform over {16, 64, 256}, a preset family uniform over
    diffuse / plastic / sheen / subsurface / metal / clearcoat / thin-film and a
    preset uniform within the family."""
    from .presets import FAMILIES
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, size=count))
    sizes = rng.choice([96, 256, 512, 1024], size=count, p=[0.5, 0.3, 0.15, 0.05])
    spp = rng.choice([16, 64, 256], size=count)
    fams = list(FAMILIES)
    jobs = []
    for i in range(count):
        fam = fams[int(rng.integers(0, len(fams)))]
        names = FAMILIES[fam]
        preset = names[int(rng.integers(0, len(names)))]
        jobs.append(PreviewJob(float(arrivals[i]), int(sizes[i]), int(sizes[i]), int(spp[i]), fam, preset))
    return jobs


def cornell_box_reference(width: int = 24, height: int = 24) -> Workload:
    """RenderScene.cornellBox() (Scene/RenderScene.swift:324-380)."""
    scene = RenderScene(camera=Camera((0, 1, 3.4), (0, 1, 0), vertical_field_of_view_degrees=42.0))
    white = scene.add_material(Material(base_color=(0.78, 0.78, 0.74)))
    red = scene.add_material(Material(base_color=(0.65, 0.05, 0.04)))
    green = scene.add_material(Material(base_color=(0.12, 0.45, 0.15)))
    light = scene.add_material(Material(base_color=(1, 1, 1), emission=(1, 0.86, 0.62), emission_strength=14.0))
    scene.add(Mesh.quad((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1)), white)
    scene.add(Mesh.quad((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)), white)
    scene.add(Mesh.quad((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)), white)
    scene.add(Mesh.quad((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1)), red)
    scene.add(Mesh.quad((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)), green)
    scene.add(Mesh.quad((-0.28, 1.99, -0.25), (0.28, 1.99, -0.25), (0.28, 1.99, 0.25), (-0.28, 1.99, 0.25)), light)
    return Workload("cornell-box-reference", scene,
                    RenderSettings(width=width, height=height, max_bounces=1, quality=RenderQuality.FINAL), 1)


def material_reference(width: int = 56, height: int = 56) -> Workload:
    """RenderScene.materialReference() (Scene/RenderScene.swift:383-455) with the settings of
    MaterialReferenceRenderTests.swift:11-19 (56x56, 2 bounces, final quality, 4 samples)."""
    scene = RenderScene(camera=Camera((0, 1.65, 5.2), (0, 0.75, 0), vertical_field_of_view_degrees=38.0))
    floor = scene.add_material(Material(base_color=(0.62, 0.62, 0.58)))
    back = scene.add_material(Material(base_color=(0.38, 0.42, 0.48)))
    warm = scene.add_material(Material(base_color=(0.95, 0.42, 0.24), roughness=0.8))
    cool = scene.add_material(Material(base_color=(0.18, 0.44, 0.9), roughness=0.18, metallic=1.0))
    green = scene.add_material(Material(base_color=(0.18, 0.72, 0.35), roughness=0.58, sheen=0.65,
                                         sheen_color=(0.72, 1.0, 0.82), sheen_roughness=0.72))
    violet = scene.add_material(Material(base_color=(0.62, 0.36, 0.95), roughness=0.35, metallic=0.55,
                                          specular_color=(0.85, 0.72, 1.0), index_of_refraction=1.65, clearcoat=0.35,
                                          clearcoat_roughness=0.06, clearcoat_index_of_refraction=1.55))
    bright = scene.add_material(Material(base_color=(0.95, 0.86, 0.42), roughness=0.08, metallic=1.0))
    light = scene.add_material(Material(base_color=(1, 1, 1), emission=(1, 0.9, 0.72), emission_strength=10.0))
    scene.add(Mesh.quad((-3, 0, 2.2), (3, 0, 2.2), (3, 0, -2.2), (-3, 0, -2.2)), floor)
    scene.add(Mesh.quad((-3, 0, -2.2), (3, 0, -2.2), (3, 2.8, -2.2), (-3, 2.8, -2.2)), back)
    scene.add(Mesh.quad((-0.8, 2.75, -0.6), (0.8, 2.75, -0.6), (0.8, 2.75, 0.4), (-0.8, 2.75, 0.4)), light)
    box = Mesh.box((-0.29, -0.29, -0.29), (0.29, 0.29, 0.29))  # Mesh.box(size: 0.58)
    placements = [(warm, (-1.6, 0.29, 0.15)), (cool, (-0.8, 0.29, -0.1)), (green, (0, 0.29, 0.1)),
                  (violet, (0.8, 0.29, -0.05)), (bright, (1.6, 0.29, 0.12))]
    for index, (material, position) in enumerate(placements):
        angle = float(np.float32(index) * np.float32(0.28) - np.float32(0.45))
        scene.add(box, material, Transform.translation(position) * Transform.rotation_y(angle))
    settings = RenderSettings(width=width, height=height, max_bounces=2, quality=RenderQuality.FINAL)
    return Workload("material-reference", scene, settings, 4)


def transparent_export_scene(width: int = 32, height: int = 32) -> Workload:
    """TransparentExportRenderTests.floatingQuadScene() with the test's settings (32x32, 1 bounce,
    transparent background, 1 sample).  The test leaves the quality at its default, preview, but its
    stored baseline (ReferenceMetrics/TransparentExport.json: 778 transparent, 246 opaque pixels) is a
    jittered one-sample render: pixel-centre rays (the preview kernel) cover 16 x 16 = 256 pixels of the
    quad.  The workload therefore renders at final quality, which reproduces the baseline."""
    scene = RenderScene(camera=Camera((0, 0, 3), (0, 0, 0), vertical_field_of_view_degrees=34.0))
    m = scene.add_material(Material(base_color=(0.9, 0.2, 0.1), emission=(0.9, 0.2, 0.1), emission_strength=1.0))
    scene.add(Mesh.quad((-0.45, -0.45, 0), (0.45, -0.45, 0), (0.45, 0.45, 0), (-0.45, 0.45, 0)), m)
    settings = RenderSettings(width=width, height=height, max_bounces=1, transparent_background=True,
                              quality=RenderQuality.FINAL)
    return Workload("transparent-export", scene, settings, 1)


def parity_quad_scene(width: int = 16, height: int = 16) -> Workload:
    """HardwareTraversalParityTests.parityScene (:168-183)."""
    scene = RenderScene(camera=Camera((0, 0, 2), (0, 0, 0), vertical_field_of_view_degrees=34.0))
    m = scene.add_material(Material(base_color=(0.25, 0.5, 0.75)))
    scene.add(Mesh.quad((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)), m)
    return Workload("parity-quad", scene,
                    RenderSettings(width=width, height=height, max_bounces=1, quality=RenderQuality.FINAL), 1)


def reused_mesh_instance_scene(width: int = 40, height: int = 40) -> Workload:
    """HardwareTraversalParityTests.reusedMeshInstanceScene (:185-224)."""
    scene = RenderScene(camera=Camera((0, 0.7, 3.8), (0, 0.35, 0), vertical_field_of_view_degrees=42.0))
    floor = scene.add_material(Material(base_color=(0.45, 0.47, 0.48)))
    red = scene.add_material(Material(base_color=(0.9, 0.2, 0.12)))
    blue = scene.add_material(Material(base_color=(0.16, 0.38, 0.9)))
    green = scene.add_material(Material(base_color=(0.2, 0.8, 0.32)))
    subject = Mesh.box((-0.275, -0.35, -0.225), (0.275, 0.35, 0.225))
    scene.add(Mesh.quad((-2.2, 0, 2.0), (2.2, 0, 2.0), (2.2, 0, -1.5), (-2.2, 0, -1.5)), floor)
    scene.add(subject, red, Transform.translation((-0.8, 0.35, 0)) * Transform.rotation_y(-0.25))
    scene.add(subject, blue, Transform.translation((0, 0.35, 0.02)) * Transform.rotation_y(0.12))
    scene.add(subject, green, Transform.translation((0.8, 0.35, -0.04)) * Transform.rotation_y(0.32))
    return Workload("reused-mesh-instances", scene,
                    RenderSettings(width=width, height=height, max_bounces=1, quality=RenderQuality.FINAL), 1)
