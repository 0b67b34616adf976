"""Serving: a persistent request loop over resident scenes (dk_server_*).

The reference renders one scene per `RenderSession`
(Sources/DenrimRendererKit/Renderer/RenderSession.swift); its CLI renders one
material preview per process (`denrim material <preset>`,
Sources/DenrimCLI/main.swift:133-163).  `RenderServer` keeps a preview scene
resident and renders many such jobs at once: each job brings its own
settings, camera, sample count and material table over the shared geometry,
and the server packs every admitted job's paths into one wavefront per wave.
More scenes can be made resident (`add_scene`); jobs name theirs, and each
step runs one packed wave per scene with work, overlapping on the device.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional, Sequence

import numpy as np

from . import abi, library
from .renderer import RenderOutput, RenderSettings, make_settings_struct
from .scene import AccelerationBuild, Camera, Material

GIB = 1 << 30


@dataclasses.dataclass
class ServerConfig:
    hbm_budget_bytes: int = 64 * GIB
    wave_paths: int = 1 << 24
    max_jobs_per_wave: int = 512
    max_resident_jobs: int = 4096
    samples_per_wave: int = 64
    policy: int = 1  # after the oldest running job: 0 admission order, 1 fewest remaining paths first

    def as_struct(self) -> abi.ServerConfig:
        c = abi.ServerConfig()
        c.hbm_budget_bytes = int(self.hbm_budget_bytes)
        c.wave_paths = int(self.wave_paths)
        c.max_jobs_per_wave = int(self.max_jobs_per_wave)
        c.max_resident_jobs = int(self.max_resident_jobs)
        c.samples_per_wave = int(self.samples_per_wave)
        c.policy = int(self.policy)
        return c


@dataclasses.dataclass
class JobStatus:
    job_id: int
    state: int
    samples_done: int
    samples: int
    waves: int
    submit_ms: float
    admit_ms: float
    finish_ms: float

    @property
    def latency_ms(self) -> float:
        return self.finish_ms - self.submit_ms


def material_table(materials: Sequence[Material]) -> np.ndarray:
    """GPUMaterial records of a job's table (Material.gpuMaterial, Material.swift:222-284)."""
    return np.array([m.gpu_material() for m in materials], dtype=abi.MATERIAL_DTYPE)


class RenderServer:
    """Compiled scenes resident on the GPU serving render jobs."""

    def __init__(self, build: AccelerationBuild, config: Optional[ServerConfig] = None):
        self._lib = library.load()
        self._build = build
        self.config = config or ServerConfig()
        self._handle = C.c_void_p()
        scene_struct = build.as_struct()
        cfg = self.config.as_struct()
        library.check(self._lib.dk_server_create(C.byref(scene_struct), C.byref(cfg), C.byref(self._handle)))
        self._builds = [build]
        self._jobs = {}

    def add_scene(self, build: AccelerationBuild) -> int:
        """Makes another compiled scene resident; returns the index jobs name it by."""
        scene_struct = build.as_struct()
        idx = C.c_uint32(0)
        library.check(self._lib.dk_server_add_scene(self._handle, C.byref(scene_struct), C.byref(idx)))
        self._builds.append(build)
        return idx.value

    def submit(self, settings: RenderSettings, camera: Camera, samples: int,
               materials: Optional[np.ndarray] = None, scene: int = 0) -> int:
        if not 0 <= scene < len(self._builds):
            raise ValueError("unknown scene index")
        table = np.ascontiguousarray(self._builds[scene].materials if materials is None else materials)
        assert table.dtype == abi.MATERIAL_DTYPE
        jd = abi.JobDesc()
        jd.settings = make_settings_struct(settings, camera)
        jd.samples = int(samples)
        jd.material_count = len(table)
        jd.materials = table.ctypes.data
        jd.scene = int(scene)
        jid = C.c_uint64(0)
        library.check(self._lib.dk_server_submit(self._handle, C.byref(jd), C.byref(jid)))
        self._jobs[jid.value] = (settings.width, settings.height)
        return jid.value

    def step(self) -> int:
        n = C.c_uint32(0)
        library.check(self._lib.dk_server_step(self._handle, C.byref(n)))
        return n.value

    def start(self) -> None:
        library.check(self._lib.dk_server_start(self._handle))

    def stop(self) -> None:
        library.check(self._lib.dk_server_stop(self._handle))

    def wait(self, job_id: int, timeout_s: float = 600.0) -> None:
        library.check(self._lib.dk_server_wait(self._handle, job_id, int(timeout_s * 1000)))

    def status(self, job_id: int) -> JobStatus:
        st = abi.JobStatus()
        library.check(self._lib.dk_server_job_status(self._handle, job_id, C.byref(st)))
        return JobStatus(st.job_id, st.state, st.samples_done, st.samples, st.waves, st.submit_ms, st.admit_ms,
                         st.finish_ms)

    def pixels(self, job_id: int, output: RenderOutput = RenderOutput.BEAUTY) -> np.ndarray:
        w, h = self._jobs[job_id]
        out = np.empty((h, w, 4), np.float32)
        library.check(self._lib.dk_server_read_output(self._handle, job_id, int(output), out.ctypes.data, w * h))
        return out

    def copy_output(self, job_id: int, output: RenderOutput, out, stream=None):
        """A finished job's output copied device to device into `out` (a
        contiguous float32 CUDA tensor of H*W*4 elements), ordered before later
        work on `stream` (default: torch's current stream)."""
        import torch
        w, h = self._jobs[job_id]
        if not (out.is_cuda and out.dtype == torch.float32 and out.is_contiguous() and out.numel() == w * h * 4):
            raise ValueError("copy_output needs a contiguous float32 CUDA tensor of width*height*4 elements")
        if stream is None:
            stream = torch.cuda.current_stream()
        library.check(self._lib.dk_server_copy_output(self._handle, job_id, int(output), C.c_void_p(out.data_ptr()),
                                                      w * h, C.c_void_p(stream.cuda_stream)))
        return out

    def copy_outputs(self, job_ids: Sequence[int], output: RenderOutput, out, stream=None):
        """The outputs of finished jobs of one size copied device to device
        into `out[i]` (a contiguous float32 CUDA tensor (n, H, W, 4)) in one
        call, ordered before later work on `stream`."""
        import torch
        ids = list(job_ids)
        if not ids:
            return out
        w, h = self._jobs[ids[0]]
        if any(self._jobs[j] != (w, h) for j in ids):
            raise ValueError("copy_outputs needs jobs of one size")
        if not (out.is_cuda and out.dtype == torch.float32 and out.is_contiguous() and out.numel() == len(ids) * w * h * 4):
            raise ValueError("copy_outputs needs a contiguous float32 CUDA tensor of n*width*height*4 elements")
        if stream is None:
            stream = torch.cuda.current_stream()
        arr = (C.c_uint64 * len(ids))(*ids)
        library.check(self._lib.dk_server_copy_outputs(self._handle, arr, len(ids), int(output),
                                                       C.c_void_p(out.data_ptr()), w * h, w * h * 16,
                                                       C.c_void_p(stream.cuda_stream)))
        return out

    def release(self, job_id: int) -> None:
        library.check(self._lib.dk_server_release(self._handle, job_id))

    def stats(self) -> dict:
        st = abi.ServerStats()
        library.check(self._lib.dk_server_get_stats(self._handle, C.byref(st)))
        return {name: getattr(st, name) for name, _ in abi.ServerStats._fields_}

    def close(self) -> None:
        if self._handle:
            self._lib.dk_server_destroy(self._handle)
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
