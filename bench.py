"""Benchmark: closest-hit Mrays/s on the 10.9M-triangle synthetic scene.

Workload: the 1920x1080 large scene (2048x2048 fBm heightfield + 500
instanced level-4 icospheres = 10,940,426 triangles, seed 1).  One step
traces two ray sets through the GPU BVH: the camera rays of one 1-spp frame
(jittered pixel samples) and their first-bounce cosine-weighted rays from the
primary hit points.  `value` = rays traced / device time with rays resident in
HBM; `e2e` = the same through the host-buffer C-ABI entry point
(krr_accel_trace_closest_host), host<->device copies included.

--impl reference times the CPU restatement of the path (the reference's own
implementation is OptiX-only and cannot run here) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "large_scene_10.9M_tris_1920x1080_primary+bounce"
METRIC = "Mrays/s closest-hit at 10M tris"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--node-format", default="0", choices=["auto", "0", "1"],
                    help="BVH node format: 0 compressed 80 B (default), 1 float 224 B, auto = "
                         "the faster after autotuning both (outside the timed region)")
    ap.add_argument("--nrc-res", default="480x270",
                    help="resolution of the time-to-relMSE comparison (0 = skip)")
    ap.add_argument("--views", type=int, default=64,
                    help="batched-views run: number of views (0 = skip)")
    ap.add_argument("--view-frames", type=int, default=5)
    ap.add_argument("--conv", type=int, default=0,
                    help="1: plain tracer's time to relMSE 0.01 on the Cornell and volume boxes")
    ap.add_argument("--conv-ref-spp", type=int, default=65536)
    ap.add_argument("--two-level", type=int, default=1,
                    help="1: also the scene as a two-level structure (memory, Mrays/s, updates)")
    ap.add_argument("--frame", type=int, default=1,
                    help="1: also time a 1920x1080 wavefront frame and its stages")
    ap.add_argument("--nrc-copies", type=int, default=8,
                    help="camera replicas traced per launch in the time-to-relMSE runs")
    ap.add_argument("--nrc-ref-spp", type=int, default=65536)
    ap.add_argument("--nrc-max-spp", type=int, default=65536)
    ap.add_argument("--nrc-max-seconds", type=float, default=40.0,
                    help="device-time cap per tracer in the time-to-relMSE runs")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(seed_offset: int = 0):
    from kiraray_gb300 import scenes
    from tests import helpers as H  # ray-set generators (numpy)

    sc = scenes.large_scene()
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=1 + seed_offset)
    return sc, tris, rays, H


class ClockSampler:
    """Samples the SM clock, its maximum, the power draw and the clock event
    (throttle) reasons during the timed region.  NVML (the library nvidia-smi
    reads) is polled every 2 ms so that a timed region of a few tens of ms
    still gets a median; without NVML, `nvidia-smi -lms 200` is read instead.
    Read-only: no clock or power setting is touched."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap"}

    def __init__(self, index: int, period_s: float = 0.002):
        self.index = index
        self.period = period_s
        self.rows = []          # (sm_mhz, max_mhz, reasons set)
        self.proc = None
        self.stop = threading.Event()
        self.nvml = None

    def _nvml_open(self):
        import ctypes as C
        for name in ("libnvidia-ml.so.1", "libnvidia-ml.so"):
            try:
                lib = C.CDLL(name)
                break
            except OSError:
                lib = None
        if lib is None or lib.nvmlInit_v2() != 0:
            return None
        h = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h)) != 0:
            return None
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons", None)
        return lib, h, reasons

    def _poll_nvml(self):
        import ctypes as C
        lib, h, reasons = self.nvml
        clk, mx, r = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and \
                    lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0:
                bits = r.value if reasons is not None and reasons(h, C.byref(r)) == 0 else 0
                self.rows.append((float(clk.value), float(mx.value),
                                  {n for b, n in self.REASONS.items() if bits & b}))
            time.sleep(self.period)

    def _read_smi(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                self.rows.append((float(parts[1]), float(parts[2]),
                                  {n for n, v in zip(names, parts[5:9]) if v == "Active"}))

    def __enter__(self):
        try:
            self.nvml = self._nvml_open()
        except Exception:
            self.nvml = None
        if self.nvml is not None:
            self.thread = threading.Thread(target=self._poll_nvml, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read_smi, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.stop.set()
        if self.nvml is not None:
            self.thread.join(timeout=2)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [r[0] for r in self.rows]
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(r[1] for r in self.rows),
                "reasons": sorted(set().union(*(r[2] for r in self.rows))),
                "samples": len(self.rows), "source": "nvml" if self.nvml else "nvidia-smi"}


def profile_figures():
    """Per-launch figures of the traversal kernel from the committed ncu
    counters (profiles/trace_closest_large_scene_figures.txt): DRAM bytes, L2
    bytes and executed warp instructions of the camera-ray launch, keyed
    lines `name: value`."""
    p = ROOT / "profiles" / "trace_closest_large_scene_figures.txt"
    out = {}
    if not p.exists():
        return out
    for line in p.read_text().splitlines():
        for key in ("dram_bytes_per_launch_full_size", "l2_bytes_per_launch_full_size",
                    "warp_inst_per_launch_full_size", "l2_peak_gbs"):
            if line.startswith(key + ":"):
                try:
                    out[key] = float(line.split(":", 1)[1].strip().split()[0])
                except ValueError:
                    pass
    return out


def l2_copy_gbs(dev) -> float:
    """Achievable L2 bandwidth, measured: a device-to-device copy between two
    24 MiB buffers (both resident in the 129 MB L2), read + write bytes per
    second, best of five batches of 50 copies."""
    import torch
    a = torch.empty(24 << 20, dtype=torch.uint8, device=dev)
    b = torch.empty_like(a)
    s = torch.cuda.current_stream()
    best = 0.0
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(50):
            b.copy_(a)
        e1.record(s)
        e1.synchronize()
        best = max(best, 2 * a.numel() * 50 / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return best


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


CPU_SAMPLE = 64   # the CPU arms trace 1 in 64 of each ray set


def cpu_sample(tris, rays, H, bvh):
    """The CPU arms' ray sample: 1 in 64 of the camera rays and 1 in 64 of
    their first-bounce rays (made from the oracle's hits of every camera
    ray, which equal the GPU's bit for bit, with the GPU arm's seed)."""
    hits = bvh.closest(rays)
    bounce = H.bounce_rays(tris, rays, hits, 2)
    return np.concatenate([rays[::CPU_SAMPLE], bounce[::CPU_SAMPLE]])


def cpu_rate(bvh, sample, threads: int, steps: int | None = None, seconds: float | None = None):
    """Oracle closest-hit throughput on `sample` (all rays per step), over
    `steps` steps or as many as fit in `seconds`."""
    bvh.closest(sample[:4096], threads)
    t0 = time.perf_counter()
    k = 0
    while True:
        bvh.closest(sample, threads)
        k += 1
        el = time.perf_counter() - t0
        if (steps is not None and k >= steps) or (seconds is not None and el >= seconds):
            break
    return sample.shape[0] * k / el / 1e6, k, el


def cpu_baseline(tris, rays, H, seconds: float, threads: int):
    """The oracle BVH's closest hit on the CPU arms' sample (same sample and
    code path as --impl reference)."""
    from oracle import pyoracle as O

    t0 = time.perf_counter()
    bvh = O.Bvh(tris)
    build_s = time.perf_counter() - t0
    sample = cpu_sample(tris, rays, H, bvh)
    v, k, el = cpu_rate(bvh, sample, threads, seconds=seconds)
    return {"value": v, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{sample.shape[0]} rays per pass (1-in-{CPU_SAMPLE} of the camera and "
                      f"first-bounce sets), {k} passes in {el:.1f} s; oracle BVH build "
                      f"{build_s:.1f} s not included"}


# Algorithmic HBM bytes per input item of each wavefront stage (queue
# items read and written, pixel-state read-modify-writes), from the queue
# layouts: Ray/Miss items 112 B, HitLight/Scatter 128 B, Shadow 80 B, hit
# record 16 B, pixel radiance 16 B, sampler state 16 B.
STAGE_BYTES = {
    "camera": 16 + 16 + 112,                # sampler RMW, ray push
    "trace_closest": 112 + 16 + 16 + 128,   # ray read, hit write+read, one push (BVH bytes apart)
    "handle_hit": 128 + 32,                 # hit-light item, L RMW
    "handle_miss": 112 + 32,                # miss item, L RMW
    "scatter": 128 + 32 + 80 + 112 + 8,     # scatter item, sampler RMW, shadow + ray push, index list
    "trace_shadow": 80 + 1 + 80 + 1 + 32,   # any-hit read/write, resolve read, L RMW
}


def wavefront_frame(sc, acc, peak, frames: int = 5):
    """One 1920x1080 frame of the pass (max depth 8, NEE): device time of the
    fused render(), then per stage (the stage-by-stage loop of
    integrator.cpp:223-254, same frame) items, time and achieved HBM bytes;
    and the first bounce's NEE shadow rays as an any-hit ray set."""
    import torch
    from kiraray_gb300.wavefront import WavefrontPathTracer

    pt = WavefrontPathTracer({"max_depth": sc.max_depth}, seed=1)
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    out = torch.empty((sc.height, sc.width, 4), device="cuda")
    s = torch.cuda.current_stream()
    for f in range(1, 4):
        pt.begin_frame(f, sc.camera)
        pt.render(out)
    ms = []
    for f in range(10, 10 + frames):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pt.begin_frame(f, sc.camera)
        e0.record(s)
        pt.render(out)
        e1.record(s)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    frame_ms = sorted(ms)[len(ms) // 2]
    # the same frames from the megakernel (one thread per path, no queues),
    # with the per-bounce regrouping of paths by hit class and without
    mk_ms = {}
    for reorder in (1, 0):
        pt.set_megakernel_reorder(reorder)
        mk = []
        for f in range(10, 10 + frames):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            pt.begin_frame(f, sc.camera)
            e0.record(s)
            pt.render_megakernel(out)
            e1.record(s)
            e1.synchronize()
            mk.append(e0.elapsed_time(e1))
        mk_ms[reorder] = sorted(mk)[len(mk) // 2]
    pt.set_megakernel_reorder(1)

    def stage_loop(count: bool, shadow_rays=None):
        items = {k: 0 for k in STAGE_BYTES}
        times = {k: 0.0 for k in STAGE_BYTES}
        pt.begin_frame(20, sc.camera)
        pt.reset_queues(-1)

        def run(name, fn, *a, n_items=None):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            fn(*a)
            e1.record(s)
            e1.synchronize()
            times[name] += e0.elapsed_time(e1)
            if count and n_items is not None:
                items[name] += n_items()

        n_pix = sc.width * sc.height
        run("camera", pt.generate_camera_rays, n_items=lambda: n_pix)
        for d in range(sc.max_depth + 1):
            pt.reset_queues(d)
            n_rays = pt.queue_size(d & 1) if count else 0
            run("trace_closest", pt.trace_closest, d, n_items=lambda: n_rays)
            n_hl, n_miss = (pt.queue_size(3), pt.queue_size(2)) if count else (0, 0)
            run("handle_hit", pt.handle_hit, n_items=lambda: n_hl)
            run("handle_miss", pt.handle_miss, n_items=lambda: n_miss)
            if d == sc.max_depth:
                break
            n_sc = pt.queue_size(5) if count else 0
            run("scatter", pt.generate_scatter_rays, d, n_items=lambda: n_sc)
            if count and d == 0 and shadow_rays is not None:
                shadow_rays.append(pt.queue_items(4)[:, 0:2, :].reshape(-1, 8).contiguous())
            n_sh = pt.queue_size(4) if count else 0
            run("trace_shadow", pt.trace_shadow, n_items=lambda: n_sh)
        return items, times

    shadow = []
    items, _ = stage_loop(True, shadow)
    _, times = stage_loop(False)
    stages = []
    for k in STAGE_BYTES:
        gbs = items[k] * STAGE_BYTES[k] / (times[k] / 1e3) / 1e9 if times[k] > 0 else 0.0
        stages.append({"stage": k, "items": int(items[k]), "ms": round(times[k], 3),
                       "bytes_per_item": STAGE_BYTES[k], "achieved_gbs": round(gbs, 1),
                       "frac_hbm": round(gbs / peak, 4)})
    # first-bounce NEE shadow rays as a ray set (any hit, tMax = 1)
    rs = shadow[0]
    occ = torch.empty((rs.shape[0],), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        acc.trace_any(rs, occ)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(10):
        acc.trace_any(rs, occ)
    e1.record(s)
    e1.synchronize()
    shadow_mrays = rs.shape[0] * 10 / (e0.elapsed_time(e1) / 1e3) / 1e6
    return {"resolution": f"{sc.width}x{sc.height}", "max_depth": sc.max_depth,
            "frame_ms": round(frame_ms, 3), "paths_per_s": round(sc.width * sc.height / frame_ms * 1e3),
            "megakernel_frame_ms": round(mk_ms[1], 3),
            "megakernel_frame_ms_without_reorder": round(mk_ms[0], 3),
            "stages": stages, "shadow_rays": int(rs.shape[0]), "shadow_mrays_s": round(shadow_mrays, 1),
            "note": "stage loop timed stage by stage (each with its own events); render() traces "
                    "each bounce's shadow rays with the next bounce's rays in one launch"}


def config_frames(args):
    """Frame time of the Cornell box (512x512, max depth 5) and the volume
    box (1024x1024, max depth 16) on the GPU, and the CPU restatement's time
    for the same frame estimated from a band of rows in the middle of the
    image (all host cores)."""
    if not args.frame:
        return None
    import torch
    from kiraray_gb300 import scenes
    from kiraray_gb300.wavefront import WavefrontPathTracer
    from oracle import pyoracle as O

    out = {}
    for name, sc, frac in (("cornell_box_512", scenes.cornell_box(512, 512, max_depth=5), 4),
                           ("volume_box_1024", scenes.volume_box(1024, 1024), 16)):
        params = {"max_depth": sc.max_depth}
        pt = WavefrontPathTracer(params, seed=sc.seed)
        pt.set_scene(sc)
        pt.resize(sc.width, sc.height)
        img = torch.empty((sc.height, sc.width, 4), device="cuda")
        s = torch.cuda.current_stream()
        ms = []
        for f in range(1, 9):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            pt.begin_frame(f, sc.camera)
            e0.record(s)
            pt.render(img)
            e1.record(s)
            e1.synchronize()
            if f > 3:
                ms.append(e0.elapsed_time(e1))
        gpu_ms = sorted(ms)[len(ms) // 2]
        work_order_ms = None
        if sc.media:   # the tracking kernels by work class, for comparison
            pt.set_media_order(1)
            qo = []
            for f in range(9, 14):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                pt.begin_frame(f, sc.camera)
                e0.record(s)
                pt.render(img)
                e1.record(s)
                e1.synchronize()
                qo.append(e0.elapsed_time(e1))
            work_order_ms = round(sorted(qo)[len(qo) // 2], 3)
            pt.set_media_order(0)
        n = sc.width * sc.height
        band = n // frac
        lo = (n - band) // 2 // sc.width * sc.width
        ora = O.PathTracer(sc)
        t0 = time.perf_counter()
        ora.render(params, 4, lo, lo + band)
        cpu_ms = (time.perf_counter() - t0) * 1e3 * n / band
        out[name] = {"gpu_frame_ms": round(gpu_ms, 3), "gpu_mpaths_s": round(n / gpu_ms / 1e3, 1),
                     "cpu_frame_ms_est": round(cpu_ms, 1), "cpu_cores": os.cpu_count() or 1,
                     "cpu_sample": f"rows {lo // sc.width}..{(lo + band) // sc.width} (1/{frac} of the pixels)",
                     "device_errors": pt.device_errors()}
        if work_order_ms is not None:
            out[name]["gpu_frame_ms_tracking_by_work_class"] = work_order_ms
    return out


def two_level(sc, rays, dev):
    """The scene as a two-level structure (each mesh geometry once, an
    instance tree over them) against the flattened one: memory, build time,
    closest-hit rate on the given ray sets, and the time of an instance
    update (the instance tree rebuilt) against a refit of the flattened
    tree."""
    import torch
    from kiraray_gb300.accel import Accel

    geoms, key_of, inst = [], {}, []
    for mi, xf in sc.instances:
        m = sc.meshes[mi]
        key = (id(m.positions), id(m.indices))
        if key not in key_of:
            key_of[key] = len(geoms)
            geoms.append(np.asarray(m.positions, np.float32)[np.asarray(m.indices)].reshape(-1, 9))
        inst.append((key_of[key], np.asarray(xf, np.float32)))
    t0 = time.perf_counter()
    acc = Accel.instanced(geoms, inst)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    st = acc.stats()
    out = {"geometries": len(geoms), "instances": len(inst),
           "node_bytes": st["node_bytes"], "triangle_bytes": st["triangle_bytes"],
           "build_ms_device": round(st["build_ms"], 3), "build_s_wall": round(build_s, 3)}
    stream = torch.cuda.current_stream()
    for name, r in rays.items():
        h = torch.empty((r.shape[0], 4), device=dev)
        for _ in range(3):
            acc.trace_closest(r, h)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            acc.trace_closest(r, h)
        e1.record(stream)
        e1.synchronize()
        out[f"{name}_mrays_s"] = round(r.shape[0] * 5 / e0.elapsed_time(e1) / 1e3, 1)
    xfs = np.stack([x for _, x in inst])
    ts = []
    for k in range(6):
        moved = xfs.copy()
        moved[1:, 1, 3] += 0.01 * (k + 1)   # every sphere instance moves up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        acc.update_instances(moved)
        torch.cuda.synchronize()
        ts.append((time.perf_counter() - t0) * 1e3)
    out["instance_update_ms_wall"] = round(sorted(ts[1:])[len(ts[1:]) // 2], 3)
    del acc
    torch.cuda.empty_cache()
    return out


def batched_views(args):
    """64 views, sides log-uniform in [256, 1024] (view i seeded 100 + i),
    even views on the large scene (max depth 8) and odd views on the volume
    box (max depth 16), one neural radiance cache for both, all in ONE
    wavefront: every stage of a bounce is one launch over the items of all
    views of both scenes, under a captured CUDA graph, with the launch shapes
    and queue capacity chosen by the autotuner (krr_wf_autotune).  Reports
    device time per frame, and for comparison the two scenes as two passes
    in one graph (a branch per pass, each with its own cache)."""
    if args.views <= 0:
        return None
    import torch
    from kiraray_gb300.nrc import NeuralRadianceCache
    from kiraray_gb300.profile import batched_workload
    from kiraray_gb300.wavefront import FrameGroup, WavefrontPathTracer

    big, vol, views = batched_workload(args.views)
    total = sum(v[1] * v[2] for v in views)
    stream = torch.cuda.Stream()

    def timed(fn, frames):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = []
        for f in frames:
            e0.record(stream)
            fn(f)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return sorted(ms)[len(ms) // 2]

    with torch.cuda.stream(stream):
        # one wavefront over both scenes
        pt = WavefrontPathTracer({"max_depth": 8}, seed=0)
        pt.set_scenes([big, vol])
        pt.set_scene_max_depth(1, vol.max_depth)
        pt.resize_views(views)
        lo, hi = pt.cache_box()
        pt.set_nrc(NeuralRadianceCache(lo, hi, seed=3), train=True)
        out = torch.empty((pt.n_pixels, 4), device="cuda")
        pt.begin_frame_views(1)
        pt.render_flat(out)
        tuning = pt.autotune(out, frames=2)
        pt.begin_frame_views(2)
        pt.render_flat(out)
        pt.capture_frame(out)
        for f in range(3, 6):
            pt.launch_frame(f)
        stream.synchronize()
        one = timed(pt.launch_frame, range(6, 6 + args.view_frames))
        errors = pt.device_errors()
        launch = pt.launch()
        del pt

        # the same views as two passes, one graph with a branch per pass
        passes, outs = [], []
        for sc, k in ((big, 0), (vol, 1)):
            p = WavefrontPathTracer({"max_depth": sc.max_depth}, seed=0)
            p.set_scene(sc)
            tris = sc.world_triangles().reshape(-1, 3)
            p.set_nrc(NeuralRadianceCache(tris.min(0), tris.max(0), seed=3), train=True)
            p.resize_views([v[:4] for v in views if v[4] == k])
            o = torch.empty((p.n_pixels, 4), device="cuda")
            p.begin_frame_views(1)
            p.render_flat(o)
            passes.append(p)
            outs.append(o)
        group = FrameGroup(passes, outs)
        group.capture()
        for f in range(2, 5):
            group.launch(f)
        stream.synchronize()
        grouped = timed(group.launch, range(5, 5 + args.view_frames))
        errors += sum(p.device_errors() for p in passes)
        group.close()
    return {"views": args.views, "pixels_per_frame": total, "scenes": ["large_scene", "volume_box"],
            "max_depth": {"large_scene": 8, "volume_box": vol.max_depth}, "nrc": True,
            "one_wavefront": True, "launches_per_stage_per_bounce": 1,
            "frame_ms": round(one, 3), "mpaths_per_s": round(total / one / 1e3, 1),
            "autotuner": {"block": tuning["block"], "blocks_per_sm": tuning["blocks_per_sm"],
                          "queue_capacity": tuning["queue_capacity"],
                          "wave": tuning["wave"] or total, "candidates": tuning["candidates"],
                          "frame_ms_chosen": round(tuning["frame_ms"], 3),
                          "frame_ms_defaults": round(tuning["default_frame_ms"], 3),
                          "note": "eager frames, cache not training during the trials"},
            "launch": launch,
            "frame_ms_two_passes_graph": round(grouped, 3), "device_errors": errors}


NRC_TUNED = {"learning_rate": 3e-3, "batch_size": 16384, "termination_spread": 0.05}


def plain_convergence(args, frames):
    """Plain tracer's time to relMSE 0.01 on the Cornell box (512x512, max
    depth 5) and the volume box (1024x1024, max depth 16) against an
    FP64-accumulated reference of the same tracer (--conv-ref-spp samples per
    pixel for the Cornell box, a quarter of that for the volume box), with
    the CPU restatement's time estimated as the samples per pixel the GPU
    needed times its measured frame time (`config_frames`)."""
    if not args.conv:
        return None
    import torch
    from kiraray_gb300 import scenes
    from kiraray_gb300.convergence import render_reference_views, time_to_error_views
    from kiraray_gb300.wavefront import WavefrontPathTracer

    out = {}
    for name, sc, copies, ref_spp in (("cornell_box_512", scenes.cornell_box(512, 512, max_depth=5), 4,
                                       args.conv_ref_spp),
                                      ("volume_box_1024", scenes.volume_box(1024, 1024), 1,
                                       max(1, args.conv_ref_spp // 4))):
        pt = WavefrontPathTracer({"max_depth": sc.max_depth}, seed=sc.seed)
        pt.set_scene(sc)
        t0 = time.perf_counter()
        ref = render_reference_views(pt, sc, copies, max(1, ref_spp // copies))
        torch.cuda.synchronize()
        ref_s = time.perf_counter() - t0
        res = time_to_error_views(pt, sc, ref, copies, target=0.01, max_frames=max(1, ref_spp // copies // 4),
                                  check_every=max(1, 64 // copies), max_seconds=120)
        cpu_ms = (frames or {}).get(name, {}).get("cpu_frame_ms_est")
        out[name] = {"reference_spp": max(1, ref_spp // copies) * copies, "reference_seconds": round(ref_s, 2),
                     "gpu_seconds": res["seconds"], "spp": res["spp"], "final_relmse": res["final_error"],
                     "gpu_ms_per_sample": round(res["ms_per_frame"] / copies, 4),
                     "cpu_seconds_est": (round(res["spp"] * cpu_ms / 1e3, 1)
                                         if res["seconds"] and cpu_ms else None)}
        del pt
    return out


def time_to_relmse(args):
    """Time to relMSE 0.01 of the plain tracer and of the neural-cache tracer
    on the large scene (max depth 8), against an FP64-accumulated reference
    of --nrc-ref-spp samples per pixel rendered by the plain tracer.  Each
    launch traces --nrc-copies replicas of the camera (batched views, frames
    replayed from a captured graph), so a frame adds that many samples."""
    if args.nrc_res in ("0", "", "none"):
        return None
    import torch
    from kiraray_gb300 import scenes
    from kiraray_gb300.convergence import render_reference_views, time_to_error_views
    from kiraray_gb300.nrc import NeuralRadianceCache
    from kiraray_gb300.wavefront import WavefrontPathTracer

    w, h = (int(x) for x in args.nrc_res.split("x"))
    copies = args.nrc_copies
    sc = scenes.large_scene(width=w, height=h, seed=3)
    params = {"max_depth": 8}
    plain = WavefrontPathTracer(params, seed=3)
    plain.set_scene(sc)
    t0 = time.perf_counter()
    ref = render_reference_views(plain, sc, copies, max(1, args.nrc_ref_spp // copies))
    torch.cuda.synchronize()
    ref_s = time.perf_counter() - t0
    max_frames = max(1, args.nrc_max_spp // copies)
    res_plain = time_to_error_views(plain, sc, ref, copies, target=0.01, max_frames=max_frames,
                                    check_every=8, max_seconds=args.nrc_max_seconds)
    tris = sc.world_triangles().reshape(-1, 3)

    def nrc_run(**cfg):
        pt = WavefrontPathTracer(params, seed=3)
        pt.set_scene(sc)
        cache = NeuralRadianceCache(tris.min(0), tris.max(0), seed=3, **cfg)
        pt.set_nrc(cache, train=True)
        return time_to_error_views(pt, sc, ref, copies, target=0.01, max_frames=max_frames,
                                   check_every=8, max_seconds=args.nrc_max_seconds)

    # the cache as specified (Adam lr 1e-2, 65,536 training records per frame)
    # with its two query rules: the path-spread rule (spread threshold 0.01,
    # the default) and the vertex after the first diffuse bounce (threshold
    # 0); then with the settings a sweep on this scene chose
    res_nrc = nrc_run()
    res_first = nrc_run(termination_spread=0.0)
    res_tuned = nrc_run(**NRC_TUNED)

    def extrapolated(res):
        # unbiased estimator: relMSE ~ 1/samples, so t(0.01) ~ t_final * err / 0.01
        c = res["curve"]
        if res["seconds"] or not c["data"]:
            return res["seconds"]
        return c["timepoints"][-1] * c["data"][-1] / 0.01

    out = {"resolution": f"{w}x{h}", "views_per_launch": copies,
           "reference_spp": max(1, args.nrc_ref_spp // copies) * copies,
           "reference_seconds": round(ref_s, 2), "target_relmse": 0.01,
           "plain_seconds": res_plain["seconds"], "plain_spp": res_plain["spp"],
           "plain_ms_per_frame": round(res_plain["ms_per_frame"], 3),
           "plain_final_relmse": res_plain["final_error"],
           "nrc_seconds": res_nrc["seconds"], "nrc_spp": res_nrc["spp"],
           "nrc_ms_per_frame": round(res_nrc["ms_per_frame"], 3),
           "nrc_final_relmse": res_nrc["final_error"]}
    if not res_plain["seconds"]:
        out["plain_seconds_extrapolated"] = extrapolated(res_plain)
    if res_nrc["seconds"]:
        out["nrc_time_fraction"] = res_nrc["seconds"] / (res_plain["seconds"] or
                                                         extrapolated(res_plain))
    out["query_rule"] = "path spread a > 0.01 a0 (Mueller et al. 2021)"
    out["nrc_first_diffuse_vertex"] = {
        "config": {"termination_spread": 0.0}, "seconds": res_first["seconds"], "spp": res_first["spp"],
        "ms_per_frame": round(res_first["ms_per_frame"], 3), "final_relmse": res_first["final_error"],
        "time_fraction": (res_first["seconds"] / (res_plain["seconds"] or extrapolated(res_plain))
                          if res_first["seconds"] else None)}
    out["nrc_tuned"] = {"config": NRC_TUNED, "seconds": res_tuned["seconds"], "spp": res_tuned["spp"],
                        "ms_per_frame": round(res_tuned["ms_per_frame"], 3),
                        "final_relmse": res_tuned["final_error"]}
    if res_tuned["seconds"]:
        out["nrc_tuned"]["time_fraction"] = res_tuned["seconds"] / (res_plain["seconds"] or
                                                                   extrapolated(res_plain))
    # equal-time comparison at the end of the (shorter) cache run
    tp = min(res_nrc["curve"]["timepoints"][-1], res_plain["curve"]["timepoints"][-1])

    def err_at(res):
        e = [d for t, d in zip(res["curve"]["timepoints"], res["curve"]["data"]) if t <= tp]
        return round(e[-1], 5) if e else None
    out["equal_time_seconds"] = round(tp, 3)
    out["equal_time_relmse"] = {"plain": err_at(res_plain), "nrc": err_at(res_nrc)}
    out["plain_curve_tail"] = list(zip(res_plain["curve"]["timesteps"][-3:],
                                       [round(x, 5) for x in res_plain["curve"]["data"][-3:]]))
    out["nrc_curve_tail"] = list(zip(res_nrc["curve"]["timesteps"][-3:],
                                     [round(x, 5) for x in res_nrc["curve"]["data"][-3:]]))
    return out


def run_reference(args, rank):
    if rank != 0:
        return
    sc, tris, rays, H = make_workload()
    from oracle import pyoracle as O

    threads = os.cpu_count() or 1
    bvh = O.Bvh(tris)
    sample = cpu_sample(tris, rays, H, bvh)
    per_step = int(sample.shape[0])
    for _ in range(args.warmup):
        bvh.closest(sample[:4096], threads)
    v, _, el = cpu_rate(bvh, sample, threads, steps=args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "rays_per_step": per_step,
                       "note": "CPU restatement of the path (oracle/): the reference traces "
                               "with OptiX on RT cores, which cannot be built or run here"},
            "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"{per_step} rays per step (1-in-{CPU_SAMPLE} of the "
                                       f"camera and first-bounce sets)"},
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, rank, world, local):
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from kiraray_gb300 import build
    from kiraray_gb300.accel import Accel

    build()
    sc, tris, rays_np, H = make_workload(seed_offset=rank)
    rays0 = torch.from_numpy(rays_np).to(dev)
    # node format and traversal settings for this workload (outside the timed region)
    formats = [0, 1] if args.node_format == "auto" else [int(args.node_format)]
    acc, tuning, tried = None, None, {}
    for fmt in formats:
        cand = Accel(tris, node_format=fmt)
        t = cand.autotune(rays0, repeats=2)
        tried[fmt] = t["ms"]
        if tuning is None or t["ms"] < tuning["ms"]:
            acc, tuning = cand, t
        else:
            del cand
    torch.cuda.synchronize()
    stats = acc.stats()
    hits0 = acc.trace_closest(rays0)
    torch.cuda.synchronize()
    bounce_np = H.bounce_rays(tris, rays_np, hits0.cpu().numpy(), 2 + rank)
    rays1 = torch.from_numpy(bounce_np).to(dev)
    hits1 = torch.empty((rays1.shape[0], 4), dtype=torch.float32, device=dev)
    sets = [(rays0, hits0), (rays1, hits1)]
    n_per_step = rays0.shape[0] + rays1.shape[0]

    # algorithmic bytes per ray from a counter-instrumented replay
    node_visits = tri_tests = 0
    for r, _ in sets:
        nn, nt = acc.trace_stats(r)
        node_visits += nn
        tri_tests += nt
    node_size = stats["node_bytes"] / stats["n_nodes"]
    alg_bytes = 48.0 * n_per_step + node_size * node_visits + 48.0 * tri_tests

    stream = torch.cuda.current_stream()
    clk = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        for r, h in sets:
            acc.trace_closest(r, h)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps * len(sets))]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    k = 0
    for _ in range(args.steps):
        for r, h in sets:
            ev[k][0].record(stream)
            acc.trace_closest(r, h)
            ev[k][1].record(stream)
            k += 1
    end.record(stream)
    torch.cuda.synchronize()
    clk.__exit__(None, None, None)
    if world > 1:
        torch.distributed.barrier()
    total_ms = start.elapsed_time(end)
    kern_ms = sum(a.elapsed_time(b) for a, b in ev)
    set_ms = [sum(ev[i][0].elapsed_time(ev[i][1]) for i in range(j, len(ev), len(sets)))
              for j in range(len(sets))]
    set_mrays = {name: round(r.shape[0] * args.steps / (ms / 1e3) / 1e6, 1)
                 for name, (r, _), ms in zip(("primary", "bounce"), sets, set_ms)}
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = n_per_step * args.steps * world / (total_ms / 1e3) / 1e6

    # end to end through the host-buffer entry point
    h_rays = [torch.from_numpy(rays_np).pin_memory(), torch.from_numpy(bounce_np).pin_memory()]
    h_hits = [torch.empty((x.shape[0], 4), dtype=torch.float32).pin_memory() for x in h_rays]
    for r, h in zip(h_rays, h_hits):
        acc.trace_closest_host(r, h)
    torch.cuda.synchronize()
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for r, h in zip(h_rays, h_hits):
            acc.trace_closest_host(r, h)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if world > 1:   # the slowest rank's time, as for `value`
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": n_per_step * e2e_steps * world / e2e_s / 1e6, "unit": "Mrays/s",
           "h2d_bytes_per_step": int(32 * n_per_step), "d2h_bytes_per_step": int(16 * n_per_step)}
    # e2e parity: the host path returns the same hits
    if not torch.equal(h_hits[0].view(torch.int32), hits0.cpu().view(torch.int32)):
        raise RuntimeError("host entry point hits differ from the device entry point")

    peak, peak_kind = peaks()
    launch_s = kern_ms / 1e3 / (args.steps * len(sets))
    achieved = alg_bytes / len(sets) / launch_s / 1e9
    prof = profile_figures()
    traffic = prof.get("dram_bytes_per_launch_full_size")
    l2_peak = l2_copy_gbs(dev)
    cam_launch_s = set_ms[0] / 1e3 / args.steps
    if rank != 0:
        return
    cpu = (cpu_baseline(tris, rays_np, H, args.cpu_seconds, os.cpu_count() or 1)
           if args.cpu_seconds > 0 else None)
    clocks = clk.summary()
    frame = wavefront_frame(sc, acc, peak) if args.frame else None
    two = two_level(sc, {"primary": rays0, "bounce": rays1}, dev) if args.two_level else None
    batched = batched_views(args)
    frames = config_frames(args)
    conv = plain_convergence(args, frames)
    nrc = time_to_relmse(args)
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "triangles": int(stats["n_triangles"]),
                   "rays_per_step": int(n_per_step), "primary_rays": int(rays0.shape[0]),
                   "bounce_rays": int(rays1.shape[0]),
                   "l2": "inputs larger than L2 (BVH nodes + triangles "
                         f"{(stats['node_bytes'] + stats['triangle_bytes']) / 1e6:.0f} MB)",
                   "bvh_build_ms": stats["build_ms"], "bvh_nodes": int(stats["n_nodes"]),
                   "bvh_depth": int(stats["max_depth"]),
                   "nodes_per_ray": node_visits / n_per_step, "tris_per_ray": tri_tests / n_per_step,
                   "tuning": {"refill_below": tuning["refill_below"],
                              "postpone_pct": tuning["postpone_pct"],
                              "node_format": stats["node_format"],
                              "primary_ms_by_format": tried},
                   "parallelism": f"replicas{world}"},
        "e2e": e2e,
        "gpu_launches": args.steps * len(sets),
        "roofline": {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind,
                     "note": f"issue-bound traversal (ncu: instruction issue, not DRAM or L2, is the "
                             f"limit); achieved = algorithmic bytes (48 B ray+hit + {node_size:.0f} B "
                             "per 8-wide node visit + 48 B per triangle test) per launch / launch time, "
                             "against the measured HBM copy bandwidth (of measured); those bytes are "
                             "served mostly by L1 and L2, so `l2` gives the L2 figure",
                     "l2": {"achieved_gbs": (prof["l2_bytes_per_launch_full_size"] / cam_launch_s / 1e9
                                             if "l2_bytes_per_launch_full_size" in prof else None),
                            "peak_gbs": l2_peak,
                            "peak_kind": "measured here: L2-resident device copy, read + write bytes",
                            "bytes_per_launch": prof.get("l2_bytes_per_launch_full_size"),
                            "launch": "camera rays, 2,073,600 (ncu lts__t_bytes.sum of one launch)"},
                     "issue": {"warp_inst_per_ray": (prof["warp_inst_per_launch_full_size"] /
                                                     rays0.shape[0]
                                                     if "warp_inst_per_launch_full_size" in prof
                                                     else None),
                               "nodes_per_ray": node_visits / n_per_step,
                               "tris_per_ray": tri_tests / n_per_step}},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "ray_sets_mrays_s": dict(set_mrays, **({"shadow": frame["shadow_mrays_s"]} if frame else {})),
        "wavefront_frame": frame,
        "two_level": dict(two, flattened={"node_bytes": stats["node_bytes"],
                                          "triangle_bytes": stats["triangle_bytes"],
                                          "primary_mrays_s": set_mrays["primary"],
                                          "bounce_mrays_s": set_mrays["bounce"]}) if two else None,
        "batched_views": batched,
        "config_frames": frames,
        "time_to_relmse": nrc,
        "plain_time_to_relmse": conv,
    }
    l2 = line["roofline"]["l2"]
    l2["frac"] = l2["achieved_gbs"] / l2["peak_gbs"] if l2["achieved_gbs"] else None
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
