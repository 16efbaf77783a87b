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
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def profile_traffic():
    """DRAM bytes per launch of the traversal kernel from the committed ncu
    summary (profiles/), or None."""
    p = ROOT / "profiles" / "trace_closest_large_scene.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch_full_size:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(tris, ray_sets, seconds: float, threads: int):
    """Oracle BVH closest-hit on a bounded sample of the same ray sets."""
    from oracle import pyoracle as O

    t0 = time.perf_counter()
    bvh = O.Bvh(tris)
    build_s = time.perf_counter() - t0
    sample = np.concatenate([r[::16] for r in ray_sets])
    n = 0
    t0 = time.perf_counter()
    chunk = 65536
    i = 0
    while True:
        part = sample[i:i + chunk]
        if part.shape[0] == 0:
            i = 0
            continue
        bvh.closest(part, threads)
        n += part.shape[0]
        i += chunk
        if time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    return {"value": n / el / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{n} rays (1-in-16 sample of the camera + first-bounce sets, cycled) in "
                      f"{el:.1f} s; oracle BVH build {build_s:.1f} s not included"}


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
    pt = WavefrontPathTracer(params, seed=3)
    pt.set_scene(sc)
    cache = NeuralRadianceCache(tris.min(0), tris.max(0), seed=3)
    pt.set_nrc(cache, train=True)
    res_nrc = time_to_error_views(pt, sc, ref, copies, target=0.01, max_frames=max_frames,
                                  check_every=8, max_seconds=args.nrc_max_seconds)

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
    # equal-time comparison: error of each tracer at the plain run's last time point
    tp = res_plain["curve"]["timepoints"][-1]
    nrc_at = [e for t, e in zip(res_nrc["curve"]["timepoints"], res_nrc["curve"]["data"]) if t <= tp]
    if nrc_at:
        out["equal_time_seconds"] = round(tp, 3)
        out["equal_time_relmse"] = {"plain": round(res_plain["curve"]["data"][-1], 5),
                                    "nrc": round(nrc_at[-1], 5)}
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
    prim = bvh.closest(rays[::8], threads)
    bounce = H.bounce_rays(tris, rays[::8], prim, 2)
    sample = np.concatenate([rays[::64], bounce[::8]])
    per_step = max(1, int(sample.shape[0]))
    for _ in range(args.warmup):
        bvh.closest(sample[:4096], threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bvh.closest(sample, threads)
    el = time.perf_counter() - t0
    v = per_step * args.steps / el / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "rays_per_step": per_step,
                       "note": "CPU restatement of the path (oracle/): the reference traces "
                               "with OptiX on RT cores, which cannot be built or run here"},
            "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"{per_step} rays per step (1-in-64 camera rays + "
                                       f"1-in-64 first-bounce rays)"},
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
    e2e = {"value": n_per_step * e2e_steps * world / e2e_s / 1e6, "unit": "Mrays/s",
           "h2d_bytes_per_step": int(32 * n_per_step), "d2h_bytes_per_step": int(16 * n_per_step)}
    # e2e parity: the host path returns the same hits
    if not torch.equal(h_hits[0].view(torch.int32), hits0.cpu().view(torch.int32)):
        raise RuntimeError("host entry point hits differ from the device entry point")

    peak, peak_kind = peaks()
    launch_s = kern_ms / 1e3 / (args.steps * len(sets))
    achieved = alg_bytes / len(sets) / launch_s / 1e9
    traffic = profile_traffic()
    if rank != 0:
        return
    cpu = (cpu_baseline(tris, [rays_np, bounce_np], args.cpu_seconds, os.cpu_count() or 1)
           if args.cpu_seconds > 0 else None)
    clocks = clk.summary()
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
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind,
                     "note": f"algorithmic bytes = 48 B ray+hit + {node_size:.0f} B per 8-wide node visit + "
                             "48 B per triangle test, per launch; they are served mostly by L2, "
                             "so the fraction is against the measured HBM copy bandwidth"},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "time_to_relmse": nrc,
    }
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
