"""Benchmark: camera paths per second of the GB300 path integrator vs the CPU restatement.

Workload (one step, the default): a full render of the dense-cloud configuration
(narvalengine_gb300/scenes/cloud_c4.json): 512^3 seeded simplex-fBm density grid (7 octaves,
density scale 80, albedo 0.99, HG g = 0.85), directional sun 3.0 at 30 deg elevation plus a
constant environment 0.2, 1024 x 1024 pixels x 16 spp, depth 256: 16 777 216 camera paths of
the plain integrator in the reference's semantics. The largest configuration that fits one
GPU, and the one the metric's time-to-relMSE half is quoted on. --scene medium_c2 | cornell_c1
| mesh_c3 | views_c5 runs the other configurations through the same harness.

  value   Mpaths/s of ne_render with the scene resident in HBM and the image written to
          device memory; each step timed with CUDA events on the library's stream, the
          L2 cache flushed (256 MiB write) between steps outside the timed events.
  e2e     Mpaths/s through the public C ABI with host buffers: every step uploads the
          scene from pinned host memory (ne_scene_upload), renders, and reads the image
          back to pinned host memory (ne_render), timed on the host clock.
  roofline  the path kernels against HBM bandwidth: algorithmic bytes = 32 B per trilinear
          density lookup (8 FP32 voxels) + 32 B per BVH node + 36 B per triangle test, counted
          by an instrumented run of the same kernel on the same paths, divided by the
          kernels' event-timed duration; `traffic` = DRAM bytes of one render from the ncu
          capture in profiles/traffic_<scene>.json, made at the tuning the bench runs; `l2`
          = the same bytes against the read bandwidth of an L2-resident buffer measured here.
  cpu_baseline  the CPU restatement of the reference integrator (oracle/; the reference itself
          does not build here) with every host thread, on a fixed pixel subset of the same
          workload (every k-th pixel in raster order, all spp), the scene read by the oracle's
          own reader.

--impl reference times that CPU restatement alone, one pass over the same pixel subset per
step, in a process that loads only the oracle (never the GPU library).
Under torchrun (N > 1), rank r renders samples [r*spp, (r+1)*spp) of the same image on its
own GPU (weak scaling, no collective on the data path); rank 0 reports total paths over
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
SCENES_DIR = os.path.join(ROOT, "narvalengine_gb300", "scenes")

DEFAULT_SCENE = "cloud_c4"
WORKLOADS = {
    "cloud_c4": "cloud_c4: 512^3 fBm cloud (7 octaves, scale 80, albedo 0.99, HG g=0.85), sun 3.0 @30deg + env 0.2, "
                "1024x1024x16spp, depth 256, plain integrator",
    "medium_c2": "medium_c2: 128^3 fBm grid (scale 20, albedo 0.9, HG g=0.8), sun 3.0 @30deg + env 0.2, "
                 "512x512x64spp, depth 64",
    "cornell_c1": "cornell_c1: Cornell box, 5 rectangles + 2 GGX spheres, 0.5x0.5 emitter (17,12,4), "
                  "256x256x16spp, depth 8, RR after 3",
    "mesh_c3": "mesh_c3: 1.31M-triangle displaced icosphere (1024 GGX groups) on a 10x10 ground, two emitters 10, "
               "1024x1024x32spp, depth 12, binned-SAH BVH built on the GPU at upload",
    "views_c5": "views_c5: 64 orbiting views (seeded sizes from {64,128,256,512}^2) of the 128^3 medium + the "
                "1.31M-triangle mesh (GPU binned-SAH BVH), 16 spp, depth 32, one persistent launch replayed as a CUDA "
                "graph, autotuned",
}
# CPU legs: every k-th pixel in raster order starting at pixel k // 2, all spp of each (for the
# views, every k-th pixel of every view). A regular lattice over the whole image, so its average
# path cost is the image's; k is sized for a pass of a few seconds on 16 host cores.
CPU_STRIDE = {"cloud_c4": 8, "medium_c2": 1, "cornell_c1": 1, "mesh_c3": 8, "views_c5": 8}
BYTES_PER_NODE = 32   # BVH node: two float4 (bounds + child/leaf words)
BYTES_PER_TRI = 36    # triangle: 9 FP32 vertex coordinates
BYTES_PER_LOOKUP = 32  # 8 FP32 voxels per trilinear density lookup
METRIC = "Mpaths/s (camera paths x spp per second, reference integrator semantics)"
L2_PROBE_BYTES = 48 << 20  # read-bandwidth probe buffer, well inside the 129 MB L2


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-reduction across ranks (torch.distributed when WORLD_SIZE > 1)."""

    def __init__(self, world: int, backend: str):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend=backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        if self.dist.get_backend() == "nccl":
            t = t.cuda()
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if not self.lines:
            # a timed region shorter than the sampling period: one reading right after it
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=10)
                self.lines = [ln.strip() for ln in out.stdout.splitlines() if ln.strip()]
            except (OSError, subprocess.SubprocessError):
                pass
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU legs (oracle only)
def render_params(seed: int = 0, spp: int = 0, sample_offset: int = 0, flags: int = 0):
    from narvalengine_gb300._abi import NeRenderParams  # a ctypes structure; loads no library
    p = NeRenderParams()
    p.seed, p.spp, p.bounces, p.rr, p.rr_after, p.sample_offset, p.flags = seed, spp, -1, -1, 3, sample_offset, flags
    return p


def sample_pixels(n_pixels: int, stride: int) -> np.ndarray:
    return np.arange(stride // 2, n_pixels, stride, dtype=np.uint32)


def lattice_rule(stride: int) -> str:
    return "every pixel" if stride == 1 else f"every {stride}th pixel (raster order, from pixel {stride // 2})"


class CpuWorkload:
    """The workload's fixed pixel subset on the oracle (the CPU restatement of the reference
    integrator), its scene read by the oracle's own reader."""

    def __init__(self, scene_name: str, threads: int):
        from oracle import oracle as orc
        self.name = scene_name
        self.threads = threads
        self.stride = CPU_STRIDE[scene_name]
        self.orc = orc.OracleScene.from_json(os.path.join(SCENES_DIR, scene_name + ".json"))
        self.spp = self.orc.spp
        if scene_name == "views_c5":
            from narvalengine_gb300.batch import orbit_views
            from oracle.scene_reader import camera_struct
            self.views = orbit_views(64, spp=self.spp, camera_look_at=camera_struct)
            self.keys = []
            for _, w, h, spp in self.views:
                px = sample_pixels(w * h, self.stride)
                self.keys.append(np.stack([np.repeat(px, spp), np.tile(np.arange(spp, dtype=np.uint32), len(px))], 1))
            self.paths = sum(len(k) for k in self.keys)
            self.rule = f"{lattice_rule(self.stride)} of each of the 64 views, all {self.spp} spp: {self.paths} paths per pass"
        else:
            self.pixels = sample_pixels(self.orc.width * self.orc.height, self.stride)
            self.paths = len(self.pixels) * self.spp
            self.rule = (f"{lattice_rule(self.stride)}, all {self.spp} spp: {len(self.pixels)} pixels = {self.paths} "
                         f"paths per pass")

    def one_pass(self, seed: int = 1) -> float:
        """Seconds for one pass over the subset."""
        if self.name == "views_c5":
            t0 = time.perf_counter()
            p = render_params(seed=seed)
            for v, (cam, w, h, _) in enumerate(self.views):
                self.orc.trace_view_paths(cam, w, h, v + 1, self.keys[v], p, self.threads)
            return time.perf_counter() - t0
        _, secs, _ = self.orc.render_pixel_list(render_params(seed=seed, spp=self.spp), self.pixels, self.threads)
        return secs

    def baseline(self, min_seconds: float) -> dict:
        """Passes over the subset until at least `min_seconds` of CPU work; Mpaths/s over them."""
        secs, reps = 0.0, 0
        while reps == 0 or secs < min_seconds:
            secs += self.one_pass()
            reps += 1
        return {"value": self.paths * reps / secs / 1e6, "unit": "Mpaths/s", "cores": self.threads, "kind": "port",
                "sample": f"{self.rule}; {reps} pass(es), {secs:.2f} s"}

    def close(self):
        self.orc.close()


def run_reference(args, rank: int, world: int):
    """The reference arm: the CPU restatement alone, one pass over the subset per step. The
    process loads liboracle.so only."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    w = CpuWorkload(args.scene, threads)
    for _ in range(args.warmup):
        w.one_pass()
    secs = [w.one_pass() for _ in range(args.steps)]
    total = sum(secs)
    v = w.paths * args.steps / total / 1e6
    line = {"metric": METRIC, "value": v, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "impl": "reference",
            "config": {"workload": WORKLOADS[args.scene], "sample": w.rule},
            "cpu_baseline": {"value": v, "unit": "Mpaths/s", "cores": threads, "kind": "port",
                             "sample": f"{w.rule}; one pass per step, {args.steps} steps, {total:.2f} s"},
            "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    w.close()
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU legs
def pin_scene_inputs(host):
    """Moves the scene's density grids to pinned host memory (kept alive by the returned
    tensors) and returns the bytes one upload copies: grids plus the instance, model,
    primitive, material, light and medium tables."""
    import ctypes
    import torch
    from narvalengine_gb300 import _abi
    desc = host.desc
    h2d, keep = 0, []
    for i in range(desc.n_media):
        m = desc.media[i]
        if m.type == 0:
            n = m.res[0] * m.res[1] * m.res[2]
            t = torch.empty(n, dtype=torch.float32, pin_memory=True)
            ctypes.memmove(t.data_ptr(), ctypes.addressof(m.grid.contents), n * 4)
            m.grid = ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float))
            keep.append(t)
            h2d += n * 4
    h2d += (desc.n_instances + desc.n_light_instances) * ctypes.sizeof(_abi.NeInstance) + \
        desc.n_models * ctypes.sizeof(_abi.NeModel) + desc.n_prims * ctypes.sizeof(_abi.NePrimitive) + \
        desc.n_materials * ctypes.sizeof(_abi.NeMaterial) + desc.n_lights * ctypes.sizeof(_abi.NeLight) + \
        desc.n_media * ctypes.sizeof(_abi.NeMedium) + desc.n_model_materials * 4
    return h2d, keep


def pinned_profile(scene_name: str):
    """profiles/traffic_<scene>.json: the tuning the DRAM-traffic capture was made at, and its
    bytes per render (or None)."""
    p = os.path.join(ROOT, "profiles", f"traffic_{scene_name}.json")
    if not os.path.exists(p):
        return None
    try:
        d = json.load(open(p))
        return d if "tuning" in d and "dram_bytes_per_launch" in d else None
    except Exception:
        return None


def cpu_leg(args, rank: int, world: int):
    if rank != 0 or args.no_cpu or world != 1:
        return None
    w = CpuWorkload(args.scene, os.cpu_count() or 1)
    try:
        return w.baseline(args.cpu_seconds)
    finally:
        w.close()


def run_views(args, rank: int, world: int, local: int):
    """The multi-view workload: 64 views in one launch; `value` = aggregate Mpaths/s over all
    views, with per-view completion latency (p50/p99) from the kernel's own timestamps."""
    import narvalengine_gb300 as ne
    from narvalengine_gb300.batch import orbit_views
    d = Dist(world, "nccl")
    ctx = ne.Context(local)
    host = ne.SceneHost.from_json(os.path.join(SCENES_DIR, "views_c5.json"))
    scene = ctx.upload(host)
    views = orbit_views(64, spp=host.spp)
    p = ne.render_params(seed=1 + rank)
    vb = ne.Views(scene, views, p)
    best, _ = vb.autotune(repeats=1)
    paths = sum(w * h * s for _, w, h, s in views)
    for _ in range(args.warmup):
        vb.render()
    ctx.synchronize()
    d.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms, p50, p99 = [], [], []
    launches = 0
    for _ in range(args.steps):
        ctx.flush_l2(256 << 20)
        st = vb.render()
        launches += st["kernel_launches"]
        ms.append(st["ms"])
        p50.append(st["latency_p50_ms"])
        p99.append(st["latency_p99_ms"])
    clk = clocks.stop()
    d.barrier()
    total_ms = d.max(sum(ms))
    value = paths * args.steps * world / (total_ms / 1e3) / 1e6
    # e2e: upload the scene, build the batch, render, read every image back
    out_bytes = sum(w * h * 12 for _, w, h, _ in views)
    h2d, pinned = pin_scene_inputs(host)
    d.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s2 = ctx.upload(host)
        v2 = ne.Views(s2, views, p)
        v2.set_tuning(**best)
        v2.render()
        for v in range(len(views)):
            v2.image(v)
        v2.close()
        s2.close()
    e2e_s = d.max(time.perf_counter() - t0)
    e2e = paths * args.steps * world / e2e_s / 1e6
    cpu = cpu_leg(args, rank, world)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
                "config": {"workload": WORKLOADS["views_c5"], "paths_per_step": paths, "views": len(views),
                           "l2": "flushed between steps (256 MiB write, outside events)",
                           "parallelism": f"{world} GPU(s), sample seeds per rank", "tuning": best},
                "latency_ms": {"p50": statistics.median(p50), "p99": statistics.median(p99)},
                "e2e": {"value": e2e, "unit": "Mpaths/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": out_bytes},
                "gpu_launches": launches,
                "roofline": None, "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(line), flush=True)
    vb.close()
    scene.close()
    ctx.close()
    d.close()


def run_profile_case(args):
    """Small case for ncu: the same scene at a reduced sample count, rendered twice at the
    pinned (or given) tuning; the second render is the one to capture."""
    import narvalengine_gb300 as ne
    ctx = ne.Context(0)
    host = ne.SceneHost.from_json(os.path.join(SCENES_DIR, args.scene + ".json"))
    scene = ctx.upload(host)
    apply_tuning(args, scene, host)
    for _ in range(2):
        _, st = scene.render(ne.render_params(seed=1, spp=args.profile_spp))
    _, cst = scene.render(ne.render_params(seed=1, spp=args.profile_spp, flags=ne.NE_RENDER_COUNT_WORK))
    print(json.dumps({"profile_case": {"scene": args.scene, "spp": args.profile_spp, "paths": st["paths"],
                                       "kernel_ms": st["kernel_ms"], "launches": st["kernel_launches"],
                                       "tuning": scene.tuning(), "density_lookups": cst["density_lookups"],
                                       "scene_queries": cst["scene_queries"], "bvh_nodes": cst["bvh_nodes"],
                                       "prim_tests": cst["prim_tests"]}}), flush=True)
    scene.close()
    ctx.close()


def apply_tuning(args, scene, host):
    """--kernel: that tuning; --autotune: the library's autotuner on the frame (another seed);
    otherwise the tuning pinned with the DRAM-traffic capture (profiles/traffic_<scene>.json),
    else the autotuner. Returns where the tuning came from."""
    if args.kernel >= 0:
        scene.set_tuning(kernel=args.kernel, track_share=args.track_share, split_passes=args.split_passes,
                         split_half=args.split_half, pretrace=args.pretrace)
        return "given"
    prof = pinned_profile(args.scene)
    if prof is not None and not args.autotune:
        scene.set_tuning(**prof["tuning"])
        return "pinned (profiles/traffic_%s.json)" % args.scene
    scene.autotune(repeats=2, seed=7, spp=host.spp)
    return "autotuned"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU baseline leg: passes over the pixel subset until this much CPU time")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--scene", default=DEFAULT_SCENE, choices=sorted(WORKLOADS),
                    help="workload (the default is the largest configuration that fits one GPU)")
    ap.add_argument("--kernel", type=int, default=-1,
                    help="path kernel (ne_tuning.kernel): 0 straight, 1 regrouped, 2 lane refill, 3 split; "
                         "default: the tuning pinned with the traffic capture, else the autotuner")
    ap.add_argument("--autotune", action="store_true", help="run the library's autotuner instead of the pinned tuning")
    ap.add_argument("--split-passes", type=int, default=0, help="split kernel passes (0: library default)")
    ap.add_argument("--split-half", type=int, default=1, help="split kernel: 1 = deferral every half bounce")
    ap.add_argument("--pretrace", type=int, default=0,
                    help="split kernel by bounce, scenes without media: 1 = bounce rays traced ahead of each "
                         "pass, 2 = camera rays too, 3 = the light samples' shadow rays too")
    ap.add_argument("--track-share", type=int, default=16, help="regrouped kernel tracking threshold, 32nds")
    ap.add_argument("--profile-spp", type=int, default=0,
                    help="profiling case: two renders of the workload at this spp (the second is the one to capture)")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.profile_spp > 0:
        run_profile_case(args)
        return
    if args.scene == "views_c5":
        run_views(args, rank, world, local)
        return

    import narvalengine_gb300 as ne
    d = Dist(world, "nccl")
    ctx = ne.Context(local)
    host = ne.SceneHost.from_json(os.path.join(SCENES_DIR, args.scene + ".json"))
    scene = ctx.upload(host)
    tuning_source = apply_tuning(args, scene, host)
    W, H, spp = host.width, host.height, host.spp
    paths_per_step = W * H * spp
    img_bytes = W * H * 3 * 4

    # device output buffer for the resident-input leg
    import torch
    dev_img = torch.empty(W * H * 3, dtype=torch.float32, device=f"cuda:{local}")
    base = rank * spp  # weak scaling: rank r renders samples [r*spp, (r+1)*spp)
    p = ne.render_params(seed=1, sample_offset=base, flags=ne.NE_RENDER_OUT_DEVICE)

    # work counters of one launch (instrumented kernel, outside the timed region)
    pc = ne.render_params(seed=1, sample_offset=base, flags=ne.NE_RENDER_OUT_DEVICE | ne.NE_RENDER_COUNT_WORK)
    _, cstats = scene.render(pc, out=dev_img.data_ptr())

    for _ in range(args.warmup):
        scene.render(p, out=dev_img.data_ptr())
    ctx.synchronize()
    d.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    kernel_ms, step_ms = [], []
    launches = 0
    for _ in range(args.steps):
        ctx.flush_l2(256 << 20)
        ctx.record(0)
        _, st = scene.render(p, out=dev_img.data_ptr())
        ctx.record(1)
        step_ms.append(ctx.elapsed_ms(0, 1))
        kernel_ms.append(st["kernel_ms"])
        launches += st["kernel_launches"]
    ctx.synchronize()
    clk = clocks.stop()
    local_ms = sum(step_ms)
    d.barrier()
    total_ms = d.max(local_ms)
    value = paths_per_step * args.steps * world / (total_ms / 1e3) / 1e6

    # e2e: host buffers through the public API, copies inside the timed region
    h2d, pinned_grid = pin_scene_inputs(host)
    out_host = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True).numpy()
    pe = ne.render_params(seed=1, sample_offset=base)
    for _ in range(args.warmup):  # untimed, like the resident leg's warm-up
        s2 = ctx.upload(host)
        s2.set_tuning(**scene.tuning())
        s2.render(pe, out=out_host)
        s2.close()
    d.barrier()
    gc.collect()
    gc.disable()  # the host clock times the library, not a collection of the harness's objects
    t0 = time.perf_counter()
    e2e_steps = []
    for _ in range(args.steps):
        ts = time.perf_counter()
        s2 = ctx.upload(host)
        s2.set_tuning(**scene.tuning())
        s2.render(pe, out=out_host)
        s2.close()
        e2e_steps.append(round((time.perf_counter() - ts) * 1e3, 2))
    e2e_s = time.perf_counter() - t0
    gc.enable()
    d.barrier()
    e2e_s = d.max(e2e_s)
    e2e = paths_per_step * args.steps * world / e2e_s / 1e6

    peak, peak_kind = load_peaks()
    k_ms = statistics.mean(kernel_ms)
    lookups = cstats["density_lookups"]
    alg_bytes = lookups * BYTES_PER_LOOKUP + cstats["bvh_nodes"] * BYTES_PER_NODE + cstats["prim_tests"] * BYTES_PER_TRI
    achieved = alg_bytes / (k_ms / 1e3) / 1e9
    tuning = scene.tuning()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": None,
                "kernel": {0: "k_paths (straight path kernel)", 1: "k_sched (regrouped path kernel)",
                           2: "k_lanes (lane-refill path kernel)",
                           3: "k_paths + k_resume (split path kernel, passes as in config.tuning)"}.get(
                               tuning["kernel"]),
                "algorithmic_bytes_per_launch": alg_bytes,
                "bytes_rule": "32 B per density lookup + 32 B per BVH node visit + 36 B per triangle test",
                "density_lookups_per_launch": lookups, "scene_queries_per_launch": cstats["scene_queries"],
                "bvh_nodes_per_launch": cstats["bvh_nodes"], "triangle_tests_per_launch": cstats["prim_tests"],
                "kernel_ms": k_ms}
    l2_gbs = ctx.read_bandwidth(L2_PROBE_BYTES, 10)
    roofline["l2"] = {"achieved": achieved, "peak": l2_gbs, "unit": "GB/s", "frac": achieved / l2_gbs,
                      "peak_source": "measured here: ne_measure_read_bandwidth, read-only kernel reading a 48 MiB "
                                     "(L2-resident) buffer 21 times per launch, 10 launches"}
    cell_bytes = max([(m.res[0] + 1) * (m.res[1] + 1) * (m.res[2] + 1) * BYTES_PER_LOOKUP
                      for m in host.desc.media[:host.desc.n_media] if m.type == 0] or [0])
    if lookups and cell_bytes:
        # the lookups' own ceiling: random 32-byte reads from a buffer the size of the cell array
        rate = ctx.random_read_rate(cell_bytes, 10)
        got = lookups / (k_ms / 1e3)
        roofline["gather"] = {"achieved": got, "peak": rate, "unit": "lookups/s", "frac": got / rate,
                              "buffer_bytes": cell_bytes,
                              "peak_source": "measured here: ne_measure_random_read, random 32-byte reads "
                                             "(hashed indices; best of 2, 4, 8, 16 in flight per thread) from a "
                                             "buffer the size of the scene's cell array, 10 launches each"}
    prof = pinned_profile(args.scene)
    if prof is not None:
        if prof["tuning"] == tuning:
            roofline["traffic"] = prof["dram_bytes_per_launch"]
            roofline["traffic_source"] = f"profiles/traffic_{args.scene}.json (ncu, same tuning)"
        else:
            roofline["traffic_source"] = "no capture at this tuning"

    cpu = cpu_leg(args, rank, world)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
                "config": {"workload": WORKLOADS[args.scene], "paths_per_step": paths_per_step, "pixels": [W, H],
                           "spp": spp, "bounces": host.bounces,
                           "l2": "flushed between steps (256 MiB write, outside events)",
                           "e2e_host": "Python garbage collection off in the e2e loop",
                           "parallelism": f"{world} GPU(s), sample ranges per rank",
                           "tuning": tuning, "tuning_source": tuning_source},
                "e2e": {"value": e2e, "unit": "Mpaths/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": img_bytes, "step_ms": e2e_steps},
                "gpu_launches": launches,
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(line), flush=True)
    scene.close()
    ctx.close()
    d.close()


if __name__ == "__main__":
    main()
