"""Benchmark: Mpaths/s of the progressive path tracer on one GB300.

Workload (one step = one frame): the large plain-method scene — 64 seeded
noise-displaced subdivision-5 icospheres (1,310,738 triangles with ground and
16 emissive triangles), a 2048x1024 log-normal HDRI with a 1e4x sun, mixed
diffuse / GGX metal / dielectric / clearcoat materials — rendered at 1920x1080,
64 spp, 12 bounces: 132.7 M paths per step.  A path is one pixel-sample, the
unit of the reference's pixel-samples/s (Sources/DenrimCLI/main.swift:277-279).

Printed JSON fields:
  value       device-timed Mpaths/s with the scene resident in HBM (CUDA events
              on the library's stream around every stage), max over ranks.
  e2e         the same metric through the C ABI from pinned host buffers: every
              step creates a session from the host arrays (host traversal
              build, host->device copy of the scene), renders the frame and
              reads the beauty image back.  Two sessions are in flight: the
              next step's session is created on a second host thread while the
              current step renders (the host build overlaps the GPU's work);
              `sequential` in the same object is the one-at-a-time figure.
  roofline    the HBM-bound stage's (shading's) algorithmic bytes (the reference
              algorithm's material / light / environment / path-state bytes,
              counted by the CPU oracle on a 1/64 pixel subsample and scaled)
              over its event-timed duration, against the measured HBM copy
              bandwidth; `roofline.stages` adds the traversal stages (extension,
              shadow), which run from L2: the L2 bytes they move against the L2
              read bandwidth measured in the same process.
  cpu_baseline  the reference's own kernel (PathTrace.metal compiled for the
              host from oracle/_ref; the FP32 oracle port where that is not
              built) on all host cores, on a 1/64 pixel subsample of the frame.
`--impl reference` times that CPU implementation alone on a 1/256 subsample
(the reference's Metal dispatch cannot run on this machine).  `--gpus N` runs N independent
replicas (one process per GPU, weak scaling): the path has no exchange step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Mpaths/s"
L2_FLUSH_BYTES = 512 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="large", choices=["large", "serving", "denoise"],
                    help="large: the headline path-tracing step (default); serving: the material-preview job "
                         "stream through the serving loop; denoise: U-Net training and 1080p inference")
    ap.add_argument("--jobs", type=int, default=1024, help="serving: jobs taken from the 4096-job stream")
    ap.add_argument("--serving-jobs", type=int, default=256,
                    help="jobs of the serving stream measured in the default line's `serving` object")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the default line's sdf / serving / serving_with_denoising objects")
    return ap.parse_args()


def max_over_ranks(value: float, device: str) -> float:
    """The maximum of a per-rank value over all ranks (identity when the
    process group is not initialised): the step time the job is charged."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mpaths(paths_per_rank_step: float, world: int, slowest_ms: float) -> float:
    """Replicas: every rank renders its own step; the job's throughput is all
    ranks' paths over the slowest rank's step time."""
    return paths_per_rank_step * world / (slowest_ms * 1e3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    from denrimrendererkit_gb300 import scenes
    return scenes.spheres_large(width=args.width, height=args.height, samples=args.spp)


def config(args, wl, extra=None):
    cfg = {"workload": wl.name, "scene": "64 displaced subdiv-5 icospheres + ground + 16 emissive tris, "
                                        "2048x1024 HDRI (log-normal, 1e4x sun)",
           "triangles": sum(len(i.mesh.indices) // 3 for i in wl.scene.mesh_instances),
           "resolution": [args.width, args.height],
           "spp_per_step": args.spp, "max_bounces": 12, "paths_per_step": args.width * args.height * args.spp,
           "frame_seed": 1, "sample_radiance_clamp": 0, "environment_max_radiance": 0,
           "l2": "path state (~3.5 GB) exceeds L2; a 512 MB buffer is also written between steps",
           "parallelism": "replicas"}
    cfg.update(extra or {})
    return cfg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power)}


def measured_peaks(key: str = "hbm_gbs"):
    """The measured peak `key` of MEASURED_PEAKS.json (HBM copy GB/s or dense
    bf16 TFLOP/s), else the fallback figure."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        if key in d:
            return float(d[key]), "measured"
    return (6800.0 if key == "hbm_gbs" else 1900.0), "fallback"


def profile_traffic(kernel: str):
    """dram bytes per launch of `kernel` on the bench workload, from the
    committed ncu summary (profiles/<kernel>_spheres_large.md), else None."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_spheres_large.md")
    if not os.path.exists(path):
        return None
    m = re.search(r"traffic_bytes_per_frame:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def profile_stage_figures():
    """Per-frame L2 and DRAM bytes and issue activity of the traversal stages
    from the committed ncu summary (profiles/traversal_stages_spheres_large.md:
    lines `<figure>.<stage>: value`), scaled there from a small-case capture."""
    path = os.path.join(ROOT, "profiles", "traversal_stages_spheres_large.md")
    if not os.path.exists(path):
        return {}
    return {m.group(1): float(m.group(2))
            for m in re.finditer(r"^([a-z0-9_]+\.k_[a-z_]+):\s*([0-9.eE+-]+)\s*$", open(path).read(), re.M)}


# Algorithmic bytes per unit of the reference algorithm (reference layouts):
# 48 B per BVH node visited, 192 B per triangle tested, 272 B per material
# fetch, 32+192 B per light sample, 21*8 + 4*16 B per environment sample,
# 4*16 B per environment lookup.
def algorithmic_bytes(counters: dict, env_texels: int):
    search = max(1, int(np.ceil(np.log2(max(env_texels, 2)))))
    ext = 48 * counters["nodes_ext"] + 192 * counters["tris_ext"]
    shadow = 48 * counters["nodes_shadow"] + 192 * counters["tris_shadow"]
    walks = 48 * (counters["nodes_sss"]) + 192 * counters["tris_sss"]
    shade = (272 * counters["material_fetch"] + (32 + 192) * counters["light_samples"]
             + (search * 8 + 4 * 16) * counters["env_samples"] + 4 * 16 * counters["env_lookups"] + walks)
    accum = (16 + 16 + 6 * 16) * counters["paths"]
    return {"k_extend": ext, "k_shadow": shadow, "k_shade": shade, "k_finalize": accum}


def cpu_oracle_sample(wl, build, threads=0):
    """The FP32 oracle on every 8th pixel in x and y, all spp of the step: the
    work counters behind the roofline's algorithmic bytes."""
    from oracle import oracle as orc
    orc.build()
    w, h = wl.settings.width, wl.settings.height
    ys, xs = np.meshgrid(np.arange(0, h, 8), np.arange(0, w, 8), indexing="ij")
    pixels = (ys * w + xs).reshape(-1).astype(np.uint32)
    r = orc.OracleRender(build, wl.settings, wl.scene.camera)
    t0 = time.perf_counter()
    r.render(wl.samples, pixel_list=pixels, threads=threads)
    dt = time.perf_counter() - t0
    paths = len(pixels) * wl.samples
    return paths, dt, r.counter_dict(), len(pixels)


def cpu_reference_sample(wl, build, stride, threads):
    """Times the reference's own kernel (PathTrace.metal pathTraceKernel compiled
    for the host, kind "reference") on every `stride`-th pixel in x and y, all
    spp of the step; the FP32 oracle port (kind "port") where it is not built.
    Returns (paths, seconds, kind, description)."""
    from oracle import oracle as orc
    w, h = wl.settings.width, wl.settings.height
    ys, xs = np.meshgrid(np.arange(0, h, stride), np.arange(0, w, stride), indexing="ij")
    pixels = (ys * w + xs).reshape(-1).astype(np.uint32)
    kind, what = "port", "FP32 oracle port of the reference shader"
    try:
        if orc.reference_available():
            orc.load_reference()
            kind, what = "reference", "the reference's pathTraceKernel (PathTrace.metal) compiled for the host"
    except Exception as exc:  # the generated source failed to build: fall back to the port, say so
        what = f"FP32 oracle port (reference kernel build failed: {str(exc).splitlines()[0][:120]})"
    if kind == "reference":
        r = orc.ReferenceRender(build, wl.settings, wl.scene.camera)
    else:
        orc.build()
        r = orc.OracleRender(build, wl.settings, wl.scene.camera)
    t0 = time.perf_counter()
    r.render(wl.samples, pixel_list=pixels, threads=threads)
    dt = time.perf_counter() - t0
    paths = len(pixels) * wl.samples
    desc = (f"every {stride}th pixel in x and y ({len(pixels)} px) x {wl.samples} spp = {paths} paths, {what}, "
            f"{threads} threads, {dt:.1f} s")
    return paths, dt, kind, desc


def run_reference(args, rank, world):
    if rank != 0:
        return
    from denrimrendererkit_gb300 import compile_scene
    from oracle import oracle as orc
    wl = workload(args)
    build = compile_scene(wl.scene, host_builders=orc.HostBuilders)
    threads = os.cpu_count() or 1
    times, kind, desc, paths = [], "port", "", 0
    for i in range(args.warmup + args.steps):
        paths, dt, kind, desc = cpu_reference_sample(wl, build, 16, threads)
        if i >= args.warmup:
            times.append(dt)
    value = paths * len(times) / sum(times) / 1e6
    impl = ("the reference's pathTraceKernel (PathTrace.metal) compiled for the host CPU; its Metal dispatch is "
            "unavailable on this box" if kind == "reference" else "CPU oracle port of the reference shader")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(args, wl), "implementation": impl,
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": kind, "sample": desc},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def flush_l2(buf):
    import torch
    buf.add_(1.0)
    torch.cuda.synchronize()


def run_gb300(args, rank, world, local):
    import torch

    from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, library
    from denrimrendererkit_gb300.renderer import make_settings_struct

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    renderer = DenrimRenderer(local)
    wl = workload(args)
    build = compile_scene(wl.scene)
    paths_per_step = wl.settings.width * wl.settings.height * wl.samples
    flush = torch.zeros(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---------------------------------------------------------- value ----
    session = renderer.make_session(wl.scene, wl.settings, build=build)
    for _ in range(args.warmup):
        session.render(wl.samples)
        flush_l2(flush)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    dev_ms, stage = 0.0, {"k_extend": 0.0, "k_shade": 0.0, "k_shadow": 0.0, "other": 0.0}
    launches = 0
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        session.render(wl.samples)
        st = session.stats()
        dev_ms += st.last_render_ms
        stage["k_extend"] += st.last_extend_ms
        stage["k_shade"] += st.last_shade_ms
        stage["k_shadow"] += st.last_shadow_ms
        stage["other"] += st.last_other_ms
        launches += st.last_launches
        flush_l2(flush)
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    ms_step = max_over_ranks(dev_ms / args.steps, f"cuda:{local}")
    value = whole_job_mpaths(paths_per_step, world, ms_step)
    beauty = session.pixels(RenderOutput.BEAUTY)
    session.close()

    # ------------------------------------------------------------ e2e ----
    e2e = None
    if not args.no_e2e:
        pinned = {}
        for name in ("triangles", "texture_pixels", "environment_samples", "nodes", "primitive_indices", "materials",
                     "lights", "texture_descriptors"):
            a = getattr(build, name)
            t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
            t.numpy()[:] = np.frombuffer(np.ascontiguousarray(a).tobytes(), np.uint8)
            pinned[name] = (t, t.numpy().view(a.dtype).reshape(a.shape))
        pb = type(build)(**{**build.__dict__, **{k: v[1] for k, v in pinned.items()}})
        out = torch.empty(wl.settings.width * wl.settings.height * 4 * 4, dtype=torch.uint8, pin_memory=True)
        out_np = out.numpy().view(np.float32).reshape(wl.settings.height, wl.settings.width, 4)
        h2d = sum(getattr(build, k).nbytes for k in pinned)
        d2h = out.numel()
        lib = library.load()
        from concurrent.futures import ThreadPoolExecutor
        from denrimrendererkit_gb300.renderer import RenderSession

        def make():
            return RenderSession(pb, wl.settings, wl.scene.camera)

        def finish(s):
            s.render(wl.samples)
            s.pixels(RenderOutput.BEAUTY, out=out_np)
            s.close()

        e2e_times = []
        for i in range(1 + args.steps):  # one session at a time; the first step warms up
            barrier()
            t0 = time.perf_counter()
            finish(make())
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            if i >= 1:
                e2e_times.append(dt)
            flush_l2(flush)
        seq_s = max_over_ranks(sum(e2e_times) / len(e2e_times), f"cuda:{local}")
        # Pipelined: step i + 1's session (host build + uploads) is created on
        # a second thread while step i renders; every step still creates,
        # uploads, renders and reads back.
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with ThreadPoolExecutor(1) as ex:
            nxt = ex.submit(make)
            for i in range(args.steps):
                s = nxt.result()
                if i + 1 < args.steps:
                    nxt = ex.submit(make)
                finish(s)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, f"cuda:{local}")
        e2e = {"value": paths_per_step * world / e2e_s / 1e6, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
               "sequential": {"value": paths_per_step * world / seq_s / 1e6, "ms_per_step": seq_s * 1e3},
               "note": "per step: dk_session_create from pinned host arrays (host traversal build + uploads) + "
                       "render 64 spp + beauty readback; the next step's session is created on a second host "
                       "thread while the current one renders (the first step's create is not overlapped)"}
        del lib

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
        return

    # ------------------------------------------- CPU baseline + roofline ----
    cpu = None
    roof = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        paths, dt, counters, npx = cpu_oracle_sample(wl, build, threads)
        scale = paths_per_step / paths
        alg = algorithmic_bytes(counters, build.environment_samples.shape[0])
        per_frame = {k: v * scale for k, v in alg.items()}
        rpaths, rdt, rkind, rdesc = cpu_reference_sample(wl, build, 8, threads)
        cpu = {"value": rpaths / rdt / 1e6, "unit": METRIC, "cores": threads, "kind": rkind, "sample": rdesc,
               "oracle_port_mpaths_s": paths / dt / 1e6}
        kernel_ms = {k: stage[k] / args.steps for k in ("k_extend", "k_shade", "k_shadow")}
        # The memory roofline belongs to the HBM-bound stage, shading; the
        # traversal stages run from L2 and get the L2 roofline in `stages`.
        dom = "k_shade"
        peak, kind = measured_peaks()
        achieved = per_frame[dom] / (kernel_ms[dom] * 1e-3) / 1e9
        traffic = profile_traffic(dom)
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured"
                else "fallback 6.8 TB/s", "traffic": traffic,
                "units": "achieved and traffic are per step (one frame, all launches of the stage); traffic = "
                         "DRAM read+write bytes scaled from a small-case ncu capture (profiles/<stage>_spheres_large.md)",
                "algorithmic_bytes_per_step": {k: float(v) for k, v in per_frame.items()},
                "kernel_ms_per_step": kernel_ms, "slowest_stage": max(kernel_ms, key=kernel_ms.get),
                "per_path": {k: float(v) / paths for k, v in counters.items() if k != "paths"}}
        # Per stage: the traversal stages run from L2 (nodes + triangle slots,
        # 109 MB, stay resident), so their roofline is L2 bytes moved against
        # the measured L2 read bandwidth; shading's is the HBM one above.
        figs = profile_stage_figures()
        l2_peak = library.probe_bandwidth(64 << 20, 50)
        hbm_probe = library.probe_bandwidth(4 << 30, 3)
        stages = {"k_shade": {"bound": "hbm", "achieved": achieved if dom == "k_shade" else
                              per_frame["k_shade"] / (kernel_ms["k_shade"] * 1e-3) / 1e9, "peak": peak,
                              "unit": "GB/s", "traffic": traffic, "bytes": "algorithmic (reference layouts)"}}
        stages["k_shade"]["frac"] = stages["k_shade"]["achieved"] / peak
        for name, kernels in (("k_extend", ("k_extend",)), ("k_shadow", ("k_shadow_rays", "k_shadow_layers"))):
            l2 = [figs.get(f"l2_bytes_per_frame.{k}") for k in kernels]
            if any(v is None for v in l2):
                stages[name] = {"bound": "l2", "achieved": None, "note": "no ncu summary of this stage"}
                continue
            a = sum(l2) / (kernel_ms[name] * 1e-3) / 1e9
            stages[name] = {"bound": "l2", "achieved": a, "peak": l2_peak, "unit": "GB/s", "frac": a / l2_peak,
                            "l2_bytes_per_frame": sum(l2),
                            "dram_bytes_per_frame": sum(figs.get(f"dram_bytes_per_frame.{k}", 0.0) for k in kernels),
                            "issue_active_pct": {k: figs.get(f"issue_active_pct.{k}") for k in kernels},
                            "algorithmic_bytes_per_frame": float(per_frame[name]),
                            "bytes": "L2 bytes moved (ncu lts__t_bytes, small case scaled to the frame)"}
        roof["stages"] = stages
        roof["measured_l2_read_gbs"] = l2_peak
        roof["measured_hbm_read_gbs"] = hbm_probe
        roof["stage_peaks"] = ("k_shade against MEASURED_PEAKS.json hbm_gbs; the traversal stages against the L2 "
                               "read bandwidth measured live (dk_probe_bandwidth, 64 MiB buffer)")
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(args, wl), "clocks": clk, "gpu_launches": int(launches), "e2e": e2e,
            "roofline": roof, "cpu_baseline": cpu, "wall_s_timed": wall,
            "stage_ms_per_step": {k: v / args.steps for k, v in stage.items()},
            "beauty_mean": float(beauty[..., :3].mean())}
    if not args.no_extras:
        # The other configurations, measured after the headline's timed region.
        line["sdf"] = sdf_measure(args, flush)
        res, cfg = serving_measure(args.serving_jobs, modes=("packed", "one_job_per_wave", "session_per_job"))
        line["serving"] = {**cfg, "modes": res,
                           "images_per_s_vs_one_job_per_wave": res["packed"]["images_per_s"]
                           / res["one_job_per_wave"]["images_per_s"],
                           "images_per_s_vs_session_per_job": res["packed"]["images_per_s"]
                           / res["session_per_job"]["images_per_s"]}
        line["unet_inference"] = unet_inference_measure()
        line["serving_with_denoising"] = serving_with_denoising_measure()
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def sdf_measure(args, flush, steps=3, warmup=2):
    """The sparse-SDF configuration (32 smooth-union spheres in a 768^3 grid of
    8^3 bricks, ~3 % kept, FP16 distances; 1024^2 x 16 spp): device-timed
    Mpaths/s, the volume pass's roofline against HBM (brick-sample, cell and
    descriptor bytes of the reference algorithm, counted by the CPU oracle on
    every 16th pixel in x and y and scaled), and the same frame with FP32
    distances for comparison."""
    from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
    renderer = DenrimRenderer(0)
    out = {}
    images = {}
    for fmt in ("fp16", "fp32"):
        wl = scenes.sdf_spheres(fp16=(fmt == "fp16"))
        build = compile_scene(wl.scene)
        paths = wl.settings.width * wl.settings.height * wl.samples
        with renderer.make_session(wl.scene, wl.settings, build=build) as s:
            for _ in range(warmup):
                s.render(wl.samples)
                flush_l2(flush)
            dev = ext = shade = shadow = 0.0
            for _ in range(steps):
                s.render(wl.samples)
                st = s.stats()
                dev += st.last_render_ms
                ext += st.last_extend_ms
                shade += st.last_shade_ms
                shadow += st.last_shadow_ms
                flush_l2(flush)
            images[fmt] = (s.pixels(RenderOutput.BEAUTY), s.pixels(RenderOutput.DEPTH))
            out[fmt] = {"mpaths_s": paths * steps / (dev * 1e3), "ms_per_frame": dev / steps,
                        "extend_ms": ext / steps, "shade_ms": shade / steps, "shadow_ms": shadow / steps,
                        "bricks": int(len(build.volume_bricks)), "samples": int(len(build.volume_brick_samples)),
                        "distance_bytes": int(len(build.volume_brick_samples)) * (2 if fmt == "fp16" else 4)}
        if fmt == "fp16":
            wl16, build16 = wl, build
    # FP16 storage against FP32: the same frame (same RNG streams).
    b16, b32 = images["fp16"][0][..., :3].astype(np.float64), images["fp32"][0][..., :3].astype(np.float64)
    d16, d32 = images["fp16"][1][..., 0], images["fp32"][1][..., 0]
    out["fp16_vs_fp32"] = {"beauty_relative_rmse": float(np.sqrt(((b16 - b32) ** 2).mean()) / b32.mean()),
                           "depth_pixels_differing": int((d16 != d32).sum()),
                           "depth_max_relative_difference": float(np.max(np.abs(d16 - d32) / np.maximum(d32, 1e-6)))}
    roof = None
    if not args.no_cpu_baseline:
        from oracle import oracle as orc
        orc.build()
        w, h = wl16.settings.width, wl16.settings.height
        ys, xs = np.meshgrid(np.arange(0, h, 16), np.arange(0, w, 16), indexing="ij")
        pixels = (ys * w + xs).reshape(-1).astype(np.uint32)
        r = orc.OracleRender(build16, wl16.settings, wl16.scene.camera)
        r.render(wl16.samples, pixel_list=pixels, threads=os.cpu_count() or 1)
        c = r.counter_dict()
        sample_paths = len(pixels) * wl16.samples
        scale = w * h * wl16.samples / sample_paths
        vol_bytes = (16 * c["brick_samples"] + 4 * (c["grid_cells"] + c["macro_skips"]) + 128 * c["brick_tests"]) * scale
        peak, kind = measured_peaks()
        ext_ms = out["fp16"]["extend_ms"]
        achieved = vol_bytes / (ext_ms * 1e-3) / 1e9
        roof = {"kernel": "k_extend_volume (volume pass of the extend stage)", "bound": "hbm", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured" else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_frame": vol_bytes,
                "per_path": {k: float(v) / sample_paths for k, v in c.items()
                             if k in ("grid_cells", "macro_skips", "brick_tests", "brick_marches", "march_steps",
                                      "brick_hits", "brick_samples")},
                "units": "16 B per brick sample read, 4 B per grid or macro cell, 128 B per brick descriptor "
                         "(the reference's layouts), counted by the oracle on every 16th pixel in x and y, scaled",
                "note": "a lower bound of the memory side only: the 92 MB of FP16 samples stay in L2 and the pass "
                        "is bound by instruction issue and dependent-load latency (ncu, small case: 0.49 TB/s "
                        "of L2, 41 % issue-active at bounce 0; profiles/k_extend_volume_sdf_spheres.md)"}
    return {"workload": "sdf-spheres 768^3, 8^3 bricks (26.8 K kept, 3 %), 1024x1024 x 16 spp, 8 bounces",
            "value": out["fp16"]["mpaths_s"], "unit": METRIC, "fp16": out["fp16"], "fp32": out["fp32"],
            "fp16_vs_fp32": out["fp16_vs_fp32"], "roofline": roof,
            "note": "value: FP16 distance storage (the configuration's); fp32 is the same scene with FP32 distances"}


def serving_with_denoising_measure(target=0.02, n_scenes=4, views=8, size=256, train_steps=2500, margin=0.9):
    """Serving with denoising against plain rendering at a stated error target
    (relative RMSE of the displayed image): requests (`views` camera views of each of `n_scenes`
    held-out small-scene variants, all resident in one render server) served
    until each image's estimated relative RMSE (of the displayed image, over
    its mean) is at most `target` x `margin` (the estimate is statistical; the
    returned images must meet `target` itself, which the true errors below
    check):

    * denoised: two independent halves rendered per request, the residual
      U-Net over A, B and F, the reference-free estimate of dF; a request over
      the target doubles its samples (the fallback to more spp) until dF -- or
      the plain render -- meets it (`denoiser.serve_to_error_target`: the
      samples grow by the count that error ~ 1/sqrt(spp) predicts);
    * plain, batched: the same loop without the network (F returns once its
      own estimate meets the target);
    * plain, one session per request: the reference's way -- two
      RenderSessions per request rendering halves progressively, growing the
      same way until the estimate meets the target.
    The true error of the returned images is measured against 16384-spp
    renders (their own noise, from their two halves, subtracted)."""
    import dataclasses as dc
    import math
    import torch
    from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, compile_scene, scenes
    from denrimrendererkit_gb300.denoiser import (TrainingSet, UNet, average_planes, display, display_relative_rmse,
                                                  estimate_errors, next_sample_count, relative_rmse, render_pairs,
                                                  serve_to_error_target, train)
    from denrimrendererkit_gb300.renderer import RenderSession
    from denrimrendererkit_gb300.scene import Camera
    from denrimrendererkit_gb300.serving import RenderServer, ServerConfig
    r = DenrimRenderer(0)
    t0 = time.perf_counter()
    parts = [render_pairs(range(100 + 12 * i, 112 + 12 * i), size=size, noisy_spp=spp, target_spp=2048)
             for i, spp in enumerate((16, 64, 256, 1024))]
    data = TrainingSet(*[torch.cat([getattr(p, f) for p in parts])
                         for f in ("beauty", "albedo", "normal", "depth", "target")])
    render_s = time.perf_counter() - t0
    net = UNet(seed=2)
    t1 = time.perf_counter()
    train(net, data, steps=train_steps, batch=16, crop=128, lr=1e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    del data, parts
    # requests: views on a +-6 degree orbit of each held-out variant
    wls = [scenes.cornell_variant(3000 + k, size, size) for k in range(n_scenes)]
    builds = [compile_scene(wl.scene) for wl in wls]
    requests = []
    for si, wl in enumerate(wls):
        cam = wl.scene.camera
        eye = np.subtract(cam.origin, cam.target)
        for i in range(views):
            a = math.radians(-6.0 + 12.0 * i / max(views - 1, 1))
            c, sn = math.cos(a), math.sin(a)
            e = (eye[0] * c + eye[2] * sn, eye[1], -eye[0] * sn + eye[2] * c)
            cv = Camera(tuple(np.add(cam.target, e)), cam.target, up=cam.up,
                        vertical_field_of_view_degrees=cam.vertical_field_of_view_degrees)
            requests.append((wl.settings, cv, None, si))
    cfg = ServerConfig(wave_paths=1 << 24, max_jobs_per_wave=512, samples_per_wave=256)
    # Requests are served to an estimate 10 % under the target: the estimate is
    # statistical, and the images returned must meet the target itself.
    serve_at = target * margin
    with RenderServer(builds[0], cfg) as srv:
        for b in builds[1:]:
            srv.add_scene(b)
        serve_to_error_target(srv, net, requests[:4], size, size, target=serve_at)  # warm-up
        torch.cuda.synchronize()
        t = time.perf_counter()
        den = serve_to_error_target(srv, net, requests, size, size, target=serve_at, start_spp=16)
        torch.cuda.synchronize()
        den_s = time.perf_counter() - t
        t = time.perf_counter()
        plain = serve_to_error_target(srv, net, requests, size, size, target=serve_at, start_spp=16, denoise=False)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t
    # plain, one session per request (two half sessions, doubling)
    t = time.perf_counter()
    sess_spp = []
    for settings, cv, _, si in requests:
        st = [dc.replace(settings, frame_seed=(settings.frame_seed ^ k) & 0x7FFFFFFF) for k in (0x3A1, 0x3A2)]
        ss = [RenderSession(builds[si], x, cv) for x in st]
        n = 8  # samples per half session
        for s in ss:
            s.render(n)
        while True:
            a, b = (torch.from_numpy(s.pixels(RenderOutput.BEAUTY)).cuda() for s in ss)
            f = torch.empty_like(a)
            average_planes(a, b, f)
            e = estimate_errors(a, b, f, a, b, f, display=True)[0]
            if e.plain <= serve_at or 2 * n >= 8192:
                break
            add = min(next_sample_count(2 * n, e.plain, serve_at, step=16), 8192) // 2 - n
            for s in ss:
                s.render(add)
            n += add
        sess_spp.append(2 * n)
        for s in ss:
            s.close()
    torch.cuda.synchronize()
    sess_s = time.perf_counter() - t
    # true error of the returned images: one view per scene, against 16384-spp renders
    true_den, true_plain, lin_den, lin_plain = [], [], [], []
    for si in range(n_scenes):
        k = si * views
        settings, cv, _, _ = requests[k]
        halves = []
        for x in (0x7001, 0x7002):
            with RenderSession(builds[si], dc.replace(settings, frame_seed=(settings.frame_seed ^ x) & 0x7FFFFFFF),
                               cv) as s:
                s.render(8192)
                halves.append(torch.from_numpy(s.pixels(RenderOutput.BEAUTY)).cuda())
        ref = torch.empty_like(halves[0])
        average_planes(halves[0], halves[1], ref)
        m = float(ref[..., :3].double().mean())
        ref_var = float(((halves[0][..., :3] - halves[1][..., :3]).double() ** 2).mean() / 4) / (m * m)
        md = float(display(ref).mean())
        ref_var_d = float(((display(halves[0]) - display(halves[1])) ** 2).mean() / 4) / (md * md)
        for res, out, lin in ((den[k], true_den, lin_den), (plain[k], true_plain, lin_plain)):
            e = display_relative_rmse(res.image, ref)
            out.append(math.sqrt(max(e * e - ref_var_d, 0.0)))
            e = relative_rmse(res.image, ref)
            lin.append(math.sqrt(max(e * e - ref_var, 0.0)))
    n = len(requests)
    return {"target_relative_rmse": target, "served_to_estimate": serve_at, "requests": n,
            "image": f"{size}x{size} views ({views} per scene) of {n_scenes} held-out small-scene variants, "
                     "resident together in one render server",
            "images_per_s_denoised": n / den_s, "images_per_s_plain_batched": n / plain_s,
            "images_per_s_plain_session_per_request": n / sess_s,
            "ratio_vs_plain_session_per_request": sess_s / den_s, "ratio_vs_plain_batched": plain_s / den_s,
            "denoised_returned": sum(1 for x in den if x.denoised),
            "fallback_to_plain": sum(1 for x in den if not x.denoised),
            "spp_denoised_mean": float(np.mean([x.spp for x in den])),
            "spp_plain_batched_mean": float(np.mean([x.spp for x in plain])),
            "spp_plain_session_mean": float(np.mean(sess_spp)),
            "estimated_error_denoised": [x.estimate.denoised if x.denoised else x.estimate.plain
                                         for x in den[::views]],
            "rounds_denoised_mean": float(np.mean([x.rounds for x in den])),
            "error_domain": "relative RMSE of the displayed image (the reference's PNG tone curve, "
                            "PNGWriter.swift:182-188, before quantisation) over the mean displayed value",
            "true_error_denoised": true_den, "true_error_plain_batched": true_plain,
            "true_linear_error_denoised": lin_den, "true_linear_error_plain_batched": lin_plain,
            "true_error_note": "one view per scene against 16384-spp renders, the reference's own noise subtracted; "
                               "the high-spp GPU render stands in for the FP64 oracle (equal within 1e-6 relative "
                               "RMSE on the small configuration)",
            "train_steps": train_steps, "train_s": train_s, "training_pairs_render_s": render_s,
            "note": "per request: two independent halves, the residual U-Net over A, B and F, the reference-free "
                    "estimate; above the target the request doubles its samples (fallback to more spp)"}


def unet_inference_measure(reps=10):
    """The U-Net's forward pass at 1920x1088 (the network's padding of 1080p):
    CUDA-event time, TFLOP/s against the dense bf16 peak, per convolution path
    (3: the halo-row kernel where a layer fits, else the per-tap kernel in its
    row-tap mode; 2: the per-tap kernel alone, one stage per tap and chunk)."""
    import torch
    from denrimrendererkit_gb300 import DenrimRenderer, library
    from denrimrendererkit_gb300.denoiser import UNet, flops_per_pixel
    DenrimRenderer(0)
    lib = library.load()
    net = UNet(seed=1)
    flops = flops_per_pixel() * 1088 * 1920
    peak, kind = measured_peaks("bf16_tflops")
    out = {}
    for path in (3, 2):
        library.check(lib.dk_unet_set_conv_path(path))
        for _ in range(3):
            net.forward(1, 1088, 1920)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            net.forward(1, 1088, 1920)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[f"path{path}"] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12}
    library.check(lib.dk_unet_set_conv_path(3))
    # the convolutions alone: each layer of the pass timed by itself (CUDA events, 20 launches after 3)
    conv_ms = 0.0
    for (l, src, so, ldi, dst, do, ldo, hh, ww) in net.conv_plan(1, 1088, 1920):
        for _ in range(3):
            net._conv(l, src, so, ldi, dst, do, ldo, 1, hh, ww)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(20):
            net._conv(l, src, so, ldi, dst, do, ldo, 1, hh, ww)
        e1.record()
        torch.cuda.synchronize()
        conv_ms += e0.elapsed_time(e1) / 20
    conv_tflops = flops / (conv_ms * 1e-3) / 1e12
    err = C.c_int(0)
    library.check(lib.dk_unet_error(C.byref(err)))
    best = out["path3"]
    return {"workload": "5-level U-Net 32-64-96-128-160, one 1920x1088 image, forward", "ms": best["ms"],
            "gflop": flops / 1e9,
            "roofline": {"kernel": "k_conv3x3_halo (stacked taps) / k_conv3x3_tma (row-tap) / avgpool / upsample "
                                   "(whole forward pass)", "bound": "tensor",
                         "achieved": best["tflops"], "peak": peak, "unit": "TFLOP/s", "frac": best["tflops"] / peak,
                         "peak_source": f"{kind} (MEASURED_PEAKS.json bf16_tflops)"},
            "convolutions": {"ms": conv_ms, "tflops": conv_tflops, "frac": conv_tflops / peak,
                             "note": "the 19 convolutions of the pass, each layer timed by itself (the pass "
                                     "minus its pooling and upsampling and the gaps between launches)"},
            "per_path": out, "tensor_wait_errors": int(err.value)}


def percentile(values, q):
    v = sorted(values)
    if not v:
        return None
    k = min(len(v) - 1, max(0, int(round(q / 100.0 * (len(v) - 1)))))
    return v[k]


def serving_measure(n_jobs, modes=("packed", "packed_fifo", "one_job_per_wave", "session_per_job")):
    """Material-preview jobs arriving as a Poisson stream (200/s) through the
    serving loop: waves packing all admitted jobs (oldest first, then fewest
    remaining paths; and in admission order), one job per wave (per-job
    launches over the same resident scene), and one render session per job
    (the reference's way: RenderSession per request, the scene uploaded with
    each).  Returns (results per mode, workload description)."""
    from denrimrendererkit_gb300 import DenrimRenderer, RenderOutput, abi, compile_scene, scenes
    from denrimrendererkit_gb300.presets import PRESETS
    from denrimrendererkit_gb300.renderer import RenderQuality, RenderSettings, RenderSession
    from denrimrendererkit_gb300.serving import RenderServer, ServerConfig
    import dataclasses
    DenrimRenderer(0)
    scene = scenes.material_preview()
    build = compile_scene(scene)
    jobs = scenes.serving_jobs()[:n_jobs]
    tables = {}
    for j in jobs:
        if j.preset not in tables:
            t = build.materials.copy()
            t[1] = PRESETS[j.preset].gpu_material()
            tables[j.preset] = t
    paths = sum(j.width * j.height * j.samples for j in jobs)

    def settings_of(j):
        return RenderSettings(width=j.width, height=j.height, max_bounces=8, quality=RenderQuality.FINAL,
                              frame_seed=1)

    results = {}
    for mode in modes:
        done = {}
        t0 = time.perf_counter()
        if mode == "session_per_job":
            # Jobs in arrival order, each its own session (scene upload, traversal
            # build, render, beauty readback); latency from its arrival.
            backlog = 0
            for k, j in enumerate(jobs):
                delay = j.arrival_s - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                b = dataclasses.replace(build, materials=tables[j.preset])
                s = RenderSession(b, settings_of(j), scene.camera)
                s.render(j.samples)
                s.pixels(RenderOutput.BEAUTY)
                s.close()
                done[k] = (time.perf_counter() - t0 - j.arrival_s) * 1e3
                backlog = max(backlog, sum(1 for x in jobs if x.arrival_s <= time.perf_counter() - t0) - len(done))
            wall = time.perf_counter() - t0
            lat = [done[k] for k in range(len(jobs))]
            small = [done[k] for k in range(len(jobs)) if jobs[k].width <= 96]
            results[mode] = {"wall_s": wall, "images_per_s": len(jobs) / wall, "mpaths_s": paths / wall / 1e6,
                             "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99),
                             "p50_ms_96px_jobs": percentile(small, 50), "p99_ms_96px_jobs": percentile(small, 99),
                             "max_backlog_jobs": backlog}
            continue
        per_wave, policy = {"packed": (512, 1), "packed_fifo": (512, 0), "one_job_per_wave": (1, 0)}[mode]
        with RenderServer(build, ServerConfig(max_jobs_per_wave=per_wave, policy=policy)) as srv:
            srv.start()
            ids = []
            stop = threading.Event()

            def collect():
                k = 0
                while k < len(jobs):
                    while k >= len(ids):
                        if stop.is_set():
                            return
                        time.sleep(0.0005)
                    st = srv.status(ids[k])
                    if st.state == abi.JOB_DONE:
                        done[k] = st
                        srv.release(ids[k])
                        k += 1
                    else:
                        time.sleep(0.0005)

            th = threading.Thread(target=collect)
            th.start()
            backlog = 0
            for j in jobs:
                delay = j.arrival_s - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                ids.append(srv.submit(settings_of(j), scene.camera, j.samples, tables[j.preset]))
                backlog = max(backlog, len(ids) - len(done))
            th.join()
            wall = time.perf_counter() - t0
            stats = srv.stats()
            srv.stop()
        lat = [done[k].latency_ms for k in range(len(jobs))]
        small = [done[k].latency_ms for k in range(len(jobs)) if jobs[k].width <= 96]
        results[mode] = {"wall_s": wall, "images_per_s": len(jobs) / wall, "mpaths_s": paths / wall / 1e6,
                         "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99),
                         "p50_ms_96px_jobs": percentile(small, 50), "p99_ms_96px_jobs": percentile(small, 99),
                         "max_backlog_jobs": backlog, "waves": stats["waves"],
                         "mean_jobs_per_wave": stats["mean_jobs_in_wave"], "busy_s": stats["busy_ms"] / 1e3,
                         "gpu_launches": stats["kernel_launches"], "budget_peak_gb": stats["budget_peak_bytes"] / 1e9}
    workload = (f"material-preview stream: first {len(jobs)} of 4096 seeded jobs, Poisson 200/s, res "
                "{96,256,512,1024}^2 (50/30/15/5 %), spp {16,64,256}, 7 preset families, icosphere on a plane "
                "under the 2048x1024 HDRI")
    return results, {"workload": workload, "paths": paths,
                     "offered_load_gpaths_s": paths / max(jobs[-1].arrival_s, 1e-9) / 1e9}


def run_serving(args, rank):
    """The serving line: the material-preview job stream through the serving
    loop (see serving_measure)."""
    if rank != 0:
        return
    results, cfg = serving_measure(args.jobs)
    line = {"metric": "serving images/s", "value": results["packed"]["images_per_s"], "unit": "images/s",
            "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg, "serving": results,
            "images_per_s_vs_one_job_per_wave": results["packed"]["images_per_s"]
            / results["one_job_per_wave"]["images_per_s"],
            "images_per_s_vs_session_per_job": results["packed"]["images_per_s"]
            / results["session_per_job"]["images_per_s"]}
    print(json.dumps(line), flush=True)


def run_denoise(args, rank):
    """U-Net: training throughput on 16 x 256^2 crops, 1920x1088 inference
    time (tcgen05 convolution) against the bf16 tensor peak, and the
    equal-error sample count on held-out scene variants."""
    if rank != 0:
        return
    import torch
    from denrimrendererkit_gb300 import DenrimRenderer
    from denrimrendererkit_gb300.denoiser import (UNet, display_relative_rmse, flops_per_pixel, render_pairs,
                                                  spatial_denoise, train)
    DenrimRenderer(0)
    t0 = time.perf_counter()
    data = render_pairs(range(64), size=256, noisy_spp=4, target_spp=1024)
    held = render_pairs(range(2000, 2008), size=256, noisy_spp=4, target_spp=1024)
    render_s = time.perf_counter() - t0
    net = UNet(seed=1)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    steps = 2000
    losses = train(net, data, steps=steps, batch=16, crop=128, lr=1e-3, log_every=500)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    errs = {"noisy_4spp": [], "spatial_filter": [], "unet": []}
    for k in range(held.count):
        out = torch.empty_like(held.beauty[k])
        net.denoise(held.beauty[k], held.albedo[k], held.normal[k], held.depth[k], 256, 256, out)
        sp = torch.empty_like(out)
        spatial_denoise(held.beauty[k], held.depth[k], held.normal[k], held.albedo[k], sp, 256, 256)
        torch.cuda.synchronize()
        errs["noisy_4spp"].append(display_relative_rmse(held.beauty[k], held.target[k]))
        errs["spatial_filter"].append(display_relative_rmse(sp, held.target[k]))
        errs["unet"].append(display_relative_rmse(out, held.target[k]))
    mean = {k: float(np.mean(v)) for k, v in errs.items()}
    # plain sample count with the U-Net's error (noise error falls as 1/sqrt(spp))
    equal_spp = 4.0 * (mean["noisy_4spp"] / mean["unet"]) ** 2
    # Serving with denoising against plain rendering at the same error: one
    # held-out 256^2 variant rendered at 4 spp + U-Net, or at the plain
    # sample count with the U-Net's error (device time per image, warm).
    from denrimrendererkit_gb300 import compile_scene, scenes
    wl = scenes.cornell_variant(2000, 256, 256)
    vb = compile_scene(wl.scene)
    plain_spp = int(np.ceil(equal_spp))
    r = DenrimRenderer(0)
    out = torch.empty_like(held.beauty[0])

    def per_image(fn, reps=20):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps

    from denrimrendererkit_gb300 import RenderOutput
    from denrimrendererkit_gb300.denoiser import GraphedDenoiser
    graphed = GraphedDenoiser(net, 256, 256)
    kinds = (RenderOutput.BEAUTY, RenderOutput.ALBEDO, RenderOutput.NORMAL, RenderOutput.DEPTH)
    planes = [torch.empty(256, 256, 4, device="cuda") for _ in kinds]
    with r.make_session(wl.scene, wl.settings, build=vb) as s4, \
            r.make_session(wl.scene, wl.settings, build=vb) as sp:
        # Each image: a fresh render, its AOVs handed to the denoiser on the
        # device, the denoised image read back to the host.
        def denoised(use_graph):
            s4.reset_accumulation()
            s4.render(4)
            if use_graph:
                for k, t in zip(kinds, graphed.inputs):
                    s4.copy_output(k, t)
                return graphed.replay().cpu()
            for k, t in zip(kinds, planes):
                s4.copy_output(k, t)
            net.denoise(*planes, 256, 256, out)
            return out.cpu()

        def plain():
            sp.reset_accumulation()
            sp.render(plain_spp)
            return sp.pixels(RenderOutput.BEAUTY)

        t_denoised = per_image(lambda: denoised(False))
        t_graphed = per_image(lambda: denoised(True))
        t_plain = per_image(plain, reps=5)
        check = float((denoised(True) - denoised(False)).abs().max())
    batched = {f"batch_{n}": serve_batches_with_denoising(net, wl, vb, plain_spp, batch=n) for n in (8, 16, 32)}
    used_graph = t_graphed <= t_denoised
    t_ungraphed = t_denoised
    t_denoised = min(t_denoised, t_graphed)
    serving = {"image": "256x256 small-scene variant", "plain_spp_equal_error": plain_spp,
               "plain_ms_per_image": t_plain * 1e3, "denoised_ms_per_image": t_denoised * 1e3,
               "images_per_s_plain": 1.0 / t_plain, "images_per_s_denoised": 1.0 / t_denoised,
               "images_per_s_ratio": t_plain / t_denoised, "graphed_denoiser": bool(used_graph),
               "ungraphed_ms_per_image": t_ungraphed * 1e3, "graphed_ms_per_image": t_graphed * 1e3,
               "graphed_vs_direct_max_abs_diff": check,
               "note": "4 spp + U-Net vs plain rendering at the U-Net's display error; per image: reset, render, "
                       "AOVs copied device to device into the denoiser, result read back to the host; "
                       "sessions warm"}
    svgf = svgf_timing()
    # 1080p inference timing
    B = net.buffers(1, 1088, 1920)
    for _ in range(3):
        net.forward(1, 1088, 1920)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        net.forward(1, 1088, 1920)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 10
    flops = flops_per_pixel() * 1088 * 1920
    peak, kind = measured_peaks("bf16_tflops")
    achieved = flops / (ms * 1e-3) / 1e12
    line = {"metric": "denoiser 1080p inference ms", "value": ms, "unit": "ms", "n_gpus": 1,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "5-level U-Net 32-64-96-128-160 over beauty+albedo+normal+depth, "
                                   "1920x1088 inference; training 16 x 128^2 crops of 64 rendered 256^2 "
                                   "small-scene variants (4 spp -> 1024 spp)", "train_steps": steps},
            "roofline": {"kernel": "U-Net convolutions, pooling, upsampling (whole forward pass)", "bound": "tensor",
                         "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                         "peak_source": kind, "traffic": None, "gflop_per_inference": flops / 1e9},
            "train_step_ms": train_s / steps * 1e3, "render_pairs_s": render_s,
            "display_relative_rmse_held_out": mean, "plain_spp_with_unet_error": equal_spp,
            "serving_with_denoising": serving, "serving_with_denoising_batched": batched, "svgf": svgf,
            "losses": losses}
    print(json.dumps(line), flush=True)


def svgf_timing(width=1920, height=1080, frames=10):
    """Device time per frame of the SVGF denoiser (DenoiseSettings.appleSVGF:
    5 a-trous passes, radius 2) at 1920x1080 on synthetic AOV planes with a
    full temporal history."""
    import torch
    from denrimrendererkit_gb300.denoiser import SvgfDenoiser
    g = torch.Generator(device="cuda").manual_seed(5)
    shape = (height, width, 4)
    beauty = torch.rand(shape, generator=g, device="cuda")
    depth = torch.rand(shape, generator=g, device="cuda") * 4 + 1
    normal = torch.rand(shape, generator=g, device="cuda") * 0.2 + 0.4
    normal[..., 2] = 0.9
    normal[..., 3] = 1.0
    motion = torch.zeros(shape, device="cuda")
    motion[..., 3] = 1.0
    out = torch.empty(shape, device="cuda")
    s = SvgfDenoiser(width, height)
    for _ in range(5):
        s.denoise(beauty, depth, normal, motion, out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(frames):
        s.denoise(beauty, depth, normal, motion, out)
    e1.record()
    torch.cuda.synchronize()
    s.close()
    return {"ms_per_frame_1080p": e0.elapsed_time(e1) / frames, "launches_per_frame": 9,
            "note": "pack, temporal, variance, 5 a-trous passes, output copy; synthetic planes, history full"}


def serve_batches_with_denoising(net, wl, build, plain_spp, batch=8, batches=10):
    """Requests served in batches through the render server: `batch` views of
    one scene (cameras on a small orbit) rendered together in one wave at
    4 spp, handed to the U-Net device to device, denoised as one batch by a
    CUDA graph and read back; against the same requests rendered at the plain
    sample count with the U-Net's error and read back."""
    import math
    import torch
    from denrimrendererkit_gb300 import RenderOutput
    from denrimrendererkit_gb300.denoiser import GraphedDenoiser
    from denrimrendererkit_gb300.scene import Camera
    from denrimrendererkit_gb300.serving import RenderServer
    cam, st = wl.scene.camera, wl.settings
    W, H = st.width, st.height
    eye = np.subtract(cam.origin, cam.target)
    cams = []
    for i in range(batch):
        a = math.radians(-6.0 + 12.0 * i / max(batch - 1, 1))
        c, s = math.cos(a), math.sin(a)
        e = (eye[0] * c + eye[2] * s, eye[1], -eye[0] * s + eye[2] * c)
        cams.append(Camera(tuple(np.add(cam.target, e)), cam.target, up=cam.up,
                           vertical_field_of_view_degrees=cam.vertical_field_of_view_degrees))
    kinds = (RenderOutput.BEAUTY, RenderOutput.ALBEDO, RenderOutput.NORMAL, RenderOutput.DEPTH)
    graphed = GraphedDenoiser(net, W, H, batch=batch)
    plain_out = torch.empty((batch, H, W, 4), dtype=torch.float32, device="cuda")
    host = torch.empty((batch, H, W, 4), dtype=torch.float32).pin_memory()

    def run(server, spp, denoise):
        ids = [server.submit(st, c, spp) for c in cams]
        while server.step():
            pass
        if denoise:
            for k, t in zip(kinds, graphed.inputs):
                server.copy_outputs(ids, k, t)
            host.copy_(graphed.replay())
        else:
            server.copy_outputs(ids, RenderOutput.BEAUTY, plain_out)
            host.copy_(plain_out)
        for j in ids:
            server.release(j)
        return host

    def per_image(server, spp, denoise):
        run(server, spp, denoise)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(batches):
            run(server, spp, denoise)
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / (batches * batch)

    # Pipelined: batch b's U-Net (torch's stream) runs while batch b + 1 renders
    # (the server's stream); two graph instances alternate their input planes
    # (the server writes them from its own I/O stream) and pinned host buffers.
    graphs = [graphed, GraphedDenoiser(net, W, H, batch=batch)]
    hosts = [host, torch.empty((batch, H, W, 4), dtype=torch.float32).pin_memory()]
    freed = [None, None]

    def pipelined(server, count):
        for b in range(count):
            g, h = graphs[b % 2], hosts[b % 2]
            ids = [server.submit(st, c, 4) for c in cams]
            while server.step():
                pass
            if freed[b % 2] is not None:  # batch b - 2 has left this graph's inputs and host buffer
                freed[b % 2].synchronize()
            for k, t in zip(kinds, g.inputs):
                server.copy_outputs(ids, k, t)
            h.copy_(g.replay(), non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            freed[b % 2] = ev
            for j in ids:
                server.release(j)
        torch.cuda.synchronize()
        return hosts[(count - 1) % 2]

    with RenderServer(build) as server:
        t_den = per_image(server, 4, True)
        t_plain = per_image(server, plain_spp, False)
        pipelined(server, 2)
        t = time.perf_counter()
        last = pipelined(server, batches).clone()
        t_pipe = (time.perf_counter() - t) / (batches * batch)
        same = bool(torch.equal(last, run(server, 4, True)))
    return {"requests_per_batch": batch, "image": f"{W}x{H} views of one held-out small-scene variant",
            "denoised_ms_per_image": t_den * 1e3, "plain_ms_per_image": t_plain * 1e3,
            "plain_spp_equal_error": plain_spp, "images_per_s_denoised": 1.0 / t_den,
            "images_per_s_plain": 1.0 / t_plain, "images_per_s_ratio": t_plain / t_den,
            "pipelined": {"denoised_ms_per_image": t_pipe * 1e3, "images_per_s_denoised": 1.0 / t_pipe,
                          "images_per_s_ratio": t_plain / t_pipe, "images_equal_sequential": same,
                          "note": "batch b's U-Net overlaps batch b + 1's render (separate streams)"},
            "note": "render server: the batch's jobs share waves; 4 spp + batched U-Net (CUDA graph) vs plain "
                    "rendering at the U-Net's display error; outputs copied device to device, results read back"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload == "serving" and args.impl != "reference":
        run_serving(args, rank)
        return
    if args.workload == "denoise" and args.impl != "reference":
        run_denoise(args, rank)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gb300(args, rank, world, local)


if __name__ == "__main__":
    main()
