"""Python mirror of the reference's render API over the C ABI.

* `RenderQuality`, `RenderSettings` (Renderer/RenderSettings.swift:5-116)
* `RenderOutput` (Renderer/RenderOutput.swift:4-25)
* `DenrimRenderer.make_session` (Renderer/DenrimRenderer.swift:253-292)
* `RenderSession.render / render_next_sample / render_next_tile /
  update_camera / reset_accumulation / pixels` (Renderer/RenderSession.swift)

Every call goes through libdenrim_cuda.so; errors raise `DenrimError` with the
status code that maps onto `DenrimRendererError`.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import enum
import os
from typing import Optional, Sequence

import numpy as np

from . import abi, library
from .scene import AccelerationBuild, Camera, RenderScene, compile_scene


class RenderQuality(enum.IntEnum):
    PREVIEW = 0
    INTERACTIVE = 1
    FINAL = 2

    @property
    def default_sample_radiance_clamp(self) -> float:  # RenderSettings.swift:16-25
        return {0: 10.0, 1: 24.0, 2: 64.0}[int(self)]


class RenderOutput(enum.IntEnum):
    BEAUTY = 0
    DEPTH = 1
    NORMAL = 2
    ALBEDO = 3
    MATERIAL_ID = 4
    OBJECT_ID = 5
    MOTION_VECTOR = 6


DK_ENCODE_WORKSPACE_INTS = 4  # DK_ENCODE_WORKSPACE_BYTES / 4


class RenderDenoiser(enum.IntEnum):
    """RenderDenoiser (Denoising/Denoiser.swift:8-18)."""
    NONE = 0
    SIMPLE_SPATIAL = 1
    APPLE_SVGF = 2


@dataclasses.dataclass(frozen=True)
class DenoiseSettings:
    """DenoiseSettings (Denoising/Denoiser.swift:20-77); APPLE_SVGF runs the
    CUDA SVGF (the reference's is Apple's MPSSVGFDenoiser)."""
    denoiser: RenderDenoiser = RenderDenoiser.NONE
    radius: int = 2
    normal_sigma: float = 0.18
    depth_sigma: float = 0.03
    albedo_sigma: float = 0.25
    color_sigma: float = 1.0
    iterations: int = 3


DenoiseSettings.NONE = DenoiseSettings()
DenoiseSettings.SIMPLE_SPATIAL = DenoiseSettings(RenderDenoiser.SIMPLE_SPATIAL)
DenoiseSettings.APPLE_SVGF = DenoiseSettings(RenderDenoiser.APPLE_SVGF, radius=2, normal_sigma=0.18,
                                             depth_sigma=0.08, albedo_sigma=0.25, color_sigma=4.0, iterations=5)


def aov_ray_enabled(denoise) -> int:
    """GPURenderConstants.denoiserEnabled (RenderSession.swift:941): 1 when a
    denoiser is requested (or the bool knob is set)."""
    if isinstance(denoise, DenoiseSettings):
        return int(denoise.denoiser != RenderDenoiser.NONE)
    return int(bool(denoise))


def denoise_filter(denoise) -> Optional[DenoiseSettings]:
    """The filter a settings' `denoise` requests (None: no filtered beauty)."""
    if isinstance(denoise, DenoiseSettings) and denoise.denoiser != RenderDenoiser.NONE:
        return denoise
    return None


@dataclasses.dataclass
class RenderSettings:
    width: int = 512
    height: int = 512
    max_bounces: int = 4
    quality: RenderQuality = RenderQuality.PREVIEW  # the reference's default (RenderSettings.swift:80)
    previous_camera: Optional[Camera] = None
    transparent_background: bool = False
    shows_environment_background: bool = True
    background_color: Sequence[float] = (0.0, 0.0, 0.0)
    # DenoiseSettings (the reference's `denoise`, RenderSettings.swift:63): a
    # denoiser other than NONE traces the unjittered AOV ray and makes the
    # beauty output the filtered image; a bool enables the AOV ray alone.
    denoise: object = False
    sample_radiance_clamp: Optional[float] = None
    collects_traversal_stats: bool = False
    frame_seed: int = 0x1234ABCD  # RenderSession.swift:917
    max_samples_per_launch: int = 0
    # Ray-triangle test: False is the reference's Moller-Trumbore (bit-exact
    # parity); True the watertight test (Woop, Benthin and Wald 2013), which no
    # ray slips through at a shared edge or vertex.
    watertight: bool = False

    @property
    def resolved_sample_radiance_clamp(self) -> float:
        if self.sample_radiance_clamp is not None:
            return float(self.sample_radiance_clamp)
        return RenderQuality(self.quality).default_sample_radiance_clamp


def make_settings_struct(settings: RenderSettings, camera: Camera) -> abi.Settings:
    s = abi.Settings()
    s.width, s.height = settings.width, settings.height
    s.max_bounces = max(1, settings.max_bounces)
    s.quality = int(settings.quality)
    s.transparent_background = int(settings.transparent_background)
    s.shows_environment_background = int(settings.shows_environment_background)
    for i in range(3):
        s.background_color[i] = float(settings.background_color[i])
    s.sample_radiance_clamp_set = 1
    s.sample_radiance_clamp = settings.resolved_sample_radiance_clamp
    s.frame_seed = settings.frame_seed & 0xFFFFFFFF
    s.denoiser_enabled = aov_ray_enabled(settings.denoise)
    s.collects_traversal_stats = int(settings.collects_traversal_stats)
    s.camera = camera.gpu_camera(settings.width, settings.height)
    prev = settings.previous_camera
    s.previous_camera = s.camera if prev is None or prev is camera else prev.gpu_camera(settings.width, settings.height)
    s.max_samples_per_launch = settings.max_samples_per_launch
    s.triangle_test = 1 if settings.watertight else 0
    return s


class RenderSession:
    """A compiled scene resident on the GPU with its progressive accumulation."""

    def __init__(self, build: AccelerationBuild, settings: RenderSettings, camera: Camera):
        self._lib = library.load()
        self.settings = settings
        self.camera = camera
        self._build = build
        self._handle = C.c_void_p()
        scene_struct = build.as_struct()
        settings_struct = make_settings_struct(settings, camera)
        library.check(self._lib.dk_session_create(C.byref(scene_struct), C.byref(settings_struct),
                                                  C.byref(self._handle)))
        self._denoised = None  # filtered beauty (device tensor) while current
        self._svgf = None

    # RenderSession.ensureDenoisedBeautyIsCurrent (RenderSession.swift:1115-1165):
    # the requested filter over the session's own planes on the device, once
    # per new sample.
    def _denoised_beauty(self):
        f = denoise_filter(self.settings.denoise)
        if f is None:
            return None
        if self._denoised is not None:
            return self._denoised
        import torch
        from . import denoiser
        w, h = self.settings.width, self.settings.height
        planes = {k: self.copy_output(k, torch.empty(h, w, 4, device="cuda"))
                  for k in (RenderOutput.BEAUTY, RenderOutput.DEPTH, RenderOutput.NORMAL, RenderOutput.ALBEDO,
                            RenderOutput.MOTION_VECTOR)}
        out = torch.empty(h, w, 4, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        if f.denoiser == RenderDenoiser.SIMPLE_SPATIAL:
            denoiser.spatial_denoise(planes[RenderOutput.BEAUTY], planes[RenderOutput.DEPTH],
                                     planes[RenderOutput.NORMAL], planes[RenderOutput.ALBEDO], out, w, h,
                                     radius=f.radius, normal_sigma=f.normal_sigma, depth_sigma=f.depth_sigma,
                                     albedo_sigma=f.albedo_sigma, color_sigma=f.color_sigma,
                                     iterations=f.iterations, stream=st)
        else:
            if self._svgf is None:
                self._svgf = denoiser.SvgfDenoiser(w, h)
            self._svgf.denoise(planes[RenderOutput.BEAUTY], planes[RenderOutput.DEPTH], planes[RenderOutput.NORMAL],
                               planes[RenderOutput.MOTION_VECTOR], out, radius=f.radius,
                               normal_sigma=f.normal_sigma, depth_sigma=f.depth_sigma, color_sigma=f.color_sigma,
                               iterations=f.iterations, stream=st)
        self._denoised = out
        return out

    def _stale(self) -> None:
        self._denoised = None

    # RenderSession.render(samples:) (RenderSession.swift:1010-1017)
    def render(self, samples: int, to: Optional[str] = None) -> None:
        """RenderSession.render(samples:) and render(samples:to:) (RenderSession.swift:1010-1023):
        with `to`, the beauty output is then written as a PNG file there."""
        if samples < 0:
            raise ValueError("Invalid render scene: Sample count must not be negative.")
        self._stale()
        library.check(self._lib.dk_session_render(self._handle, samples))
        if to is not None:
            self.write_png(to)

    # RenderSession.writePNG(output:to:) (RenderSession.swift:1026-1034)
    def write_png(self, path: str, output: "RenderOutput" = None) -> None:
        output = RenderOutput.BEAUTY if output is None else output
        if output == RenderOutput.BEAUTY and denoise_filter(self.settings.denoise) is not None:
            w, h = self.settings.width, self.settings.height
            rgba = np.ascontiguousarray(self.rgba8(output))
            library.check(self._lib.dk_write_png(os.fsencode(path), rgba.ctypes.data, w, h))
            return
        library.check(self._lib.dk_session_write_png(self._handle, int(output), os.fsencode(path)))

    def rgba8(self, output: "RenderOutput" = None) -> np.ndarray:
        """The output as the reference's PNG export shows it (PNGWriter.visualizedRGBA8Pixels,
        Image/PNGWriter.swift:35-53), encoded on the device: uint8 (height, width, 4)."""
        output = RenderOutput.BEAUTY if output is None else output
        w, h = self.settings.width, self.settings.height
        out = np.empty((h, w, 4), np.uint8)
        den = self._denoised_beauty() if output == RenderOutput.BEAUTY else None
        if den is not None:
            import torch
            dev = torch.empty(h * w * 4, dtype=torch.uint8, device="cuda")
            ws = torch.zeros(DK_ENCODE_WORKSPACE_INTS, dtype=torch.int32, device="cuda")
            library.check(self._lib.dk_encode_rgba8(C.c_void_p(den.data_ptr()), w, h, int(output),
                                                    C.c_void_p(dev.data_ptr()), C.c_void_p(ws.data_ptr()),
                                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            out[...] = dev.cpu().numpy().reshape(h, w, 4)
            return out
        library.check(self._lib.dk_session_read_rgba8(self._handle, int(output), out.ctypes.data, out.size))
        return out

    def render_next_sample(self) -> None:
        self.render(1)

    # RenderSession.renderNextTile(_:completesSample:) (RenderSession.swift:875-889)
    def render_next_tile(self, x: int, y: int, width: int, height: int, completes_sample: bool) -> None:
        self._stale()
        library.check(self._lib.dk_session_render_tile(self._handle, x, y, width, height, int(completes_sample)))

    # RenderSession.updateCamera(_:previousCamera:) (RenderSession.swift:595-608)
    def update_camera(self, camera: Camera, previous_camera: Optional[Camera] = None) -> None:
        cur = camera.gpu_camera(self.settings.width, self.settings.height)
        prev = (previous_camera or self.camera).gpu_camera(self.settings.width, self.settings.height)
        self._stale()
        if self._svgf is not None:  # updateCamera resets accumulation (RenderSession.swift:594-608)
            self._svgf.reset()
        library.check(self._lib.dk_session_update_camera(self._handle, C.byref(cur), C.byref(prev)))
        self.camera = camera

    def reset_accumulation(self) -> None:
        self._stale()
        if self._svgf is not None:  # RenderSession.resetAccumulation (RenderSession.swift:581-587)
            self._svgf.reset()
        library.check(self._lib.dk_session_reset(self._handle))

    @property
    def sample_count(self) -> int:
        n = C.c_uint32(0)
        library.check(self._lib.dk_session_sample_count(self._handle, C.byref(n)))
        return n.value

    def stats(self) -> abi.Stats:
        st = abi.Stats()
        library.check(self._lib.dk_session_stats(self._handle, C.byref(st)))
        return st

    # RenderSession.sdfTraversalStats() / resetSDFTraversalStats() (RenderSession.swift:808-831, :611-614):
    # the SDF traversal counters of a session made with `collects_traversal_stats`, by the
    # reference's names (all zero otherwise).
    SDF_COUNTER_NAMES = ("dense_volume_tests", "dense_march_steps", "sparse_grid_cells_visited",
                         "sparse_grid_macro_skips", "sparse_brick_tests", "sparse_brick_invalid",
                         "sparse_brick_range_culls", "sparse_brick_marches", "sparse_brick_march_steps",
                         "sparse_brick_hits", "primary_scene_queries", "bounce_scene_queries",
                         "shadow_scene_queries")

    def sdf_traversal_stats(self) -> dict:
        st = self.stats()
        d = {k: int(st.sdf_counters[i]) for i, k in enumerate(self.SDF_COUNTER_NAMES)}
        # derived as RenderSession.swift:819 does: cells visited without a brick test
        d["sparse_grid_empty_cells"] = d["sparse_grid_cells_visited"] - min(d["sparse_grid_cells_visited"],
                                                                            d["sparse_brick_tests"])
        return d

    def reset_sdf_traversal_stats(self) -> None:
        library.check(self._lib.dk_session_reset_sdf_stats(self._handle))

    # RenderSession.pixels(for:) (RenderSession.swift:1037-1039): (H, W, 4) float32
    def pixels(self, output: RenderOutput = RenderOutput.BEAUTY, out: Optional[np.ndarray] = None) -> np.ndarray:
        w, h = self.settings.width, self.settings.height
        if out is None:
            out = np.empty((h, w, 4), np.float32)
        assert out.dtype == np.float32 and out.flags["C_CONTIGUOUS"] and out.size == w * h * 4
        den = self._denoised_beauty() if output == RenderOutput.BEAUTY else None
        if den is not None:  # texture(for: .beauty) is the denoised image (RenderSession.swift:1072-1080)
            out[...] = den.cpu().numpy().reshape(out.shape)
            return out
        library.check(self._lib.dk_session_read_output(self._handle, int(output), out.ctypes.data, w * h))
        return out

    # RenderSession.texture(for:) (RenderSession.swift:1072-1094): the output
    # copied device to device into `out`, a float32 CUDA tensor of H*W*4
    # elements; ordered before later work on `stream` (default: torch's
    # current stream), with no host round trip.
    def copy_output(self, output: RenderOutput, out, stream=None):
        import torch
        w, h = self.settings.width, self.settings.height
        if not (out.is_cuda and out.dtype == torch.float32 and out.is_contiguous() and out.numel() == w * h * 4):
            raise ValueError("copy_output needs a contiguous float32 CUDA tensor of width*height*4 elements")
        if stream is None:
            stream = torch.cuda.current_stream()
        library.check(self._lib.dk_session_copy_output(self._handle, int(output), C.c_void_p(out.data_ptr()), w * h,
                                                       C.c_void_p(stream.cuda_stream)))
        return out

    def close(self) -> None:
        if getattr(self, "_svgf", None) is not None:
            self._svgf.close()
            self._svgf = None
        self._denoised = None
        if self._handle:
            self._lib.dk_session_destroy(self._handle)
            self._handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class DenrimRenderer:
    """Entry point (Renderer/DenrimRenderer.swift:28-292) for CUDA sessions."""

    def __init__(self, device: int = 0):
        lib = library.load()
        library.check(lib.dk_device_open(device))
        self.device = device

    def make_session(self, scene: RenderScene, settings: RenderSettings,
                     build: Optional[AccelerationBuild] = None) -> RenderSession:
        if settings.width <= 0 or settings.height <= 0:
            raise library.DenrimError(3, "Invalid render scene: Render dimensions must be positive.")
        build = build or compile_scene(scene)
        return RenderSession(build, settings, scene.camera)
