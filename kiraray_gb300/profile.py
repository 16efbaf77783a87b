"""Fixed workloads for profiling the pass under a profiler (ncu launch lists
and single-kernel captures); prints the device time of each repetition.

    python -m kiraray_gb300.profile trace [--reps 4] [--builder 0] [--levels 2]
        closest hits of the 1920x1080 camera rays of the 10.9M-triangle scene
        (BVH builder as krr_set_bvh_builder; --levels 2: the two-level
        structure, per-geometry trees and an instance tree)
    python -m kiraray_gb300.profile cache [--configs JSON] [--res 480x270]
        relMSE curves (2k-32k samples per pixel, 8 replica views per launch)
        of the neural-cache tracer on the large scene for cache configurations
    python -m kiraray_gb300.profile update [--reps 5]
        an instance update of the large scene (re-flatten + BVH refit) against
        a full BVH rebuild, host wall time per call
    python -m kiraray_gb300.profile frame [--scene large] [--res 480x270] [--views 8] [--nrc]
                                          [--frames 3] [--seed 3] [--camera-order 1]
        frames of the wavefront pass on the large scene (max depth 8), the
        Cornell box (5) or the volume box (16), the camera replicated into
        `views` batched views, optionally with the neural radiance cache
        attached and training
    python -m kiraray_gb300.profile batched [--frames 3] [--views 64]
        eager frames of the batched configuration: 64 views of uneven sizes
        on the large scene and the volume box in one wavefront, the neural
        radiance cache attached and training
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import torch


def _timed(fn) -> float:
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    fn()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1)


def trace(reps: int, builder: int = 2, levels: int = 1) -> dict:
    import numpy as np

    from . import scenes
    from .accel import Accel, set_builder

    sc = scenes.large_scene()
    set_builder(builder)
    if levels == 2:
        # each mesh geometry once, an instance tree over them
        geoms, key_of, inst = [], {}, []
        for mi, xf in sc.instances:
            m = sc.meshes[mi]
            key = (id(m.positions), id(m.indices))
            if key not in key_of:
                key_of[key] = len(geoms)
                geoms.append(np.asarray(m.positions, np.float32)[np.asarray(m.indices)].reshape(-1, 9))
            inst.append((key_of[key], np.asarray(xf, np.float32)))
        acc = Accel.instanced(geoms, inst)
    else:
        acc = Accel(sc.world_triangles())
    set_builder(2)
    rays = torch.from_numpy(scenes.pinhole_rays(sc)).cuda()
    ms = [_timed(lambda: acc.trace_closest(rays)) for _ in range(reps)]
    return {"workload": "trace", "levels": levels, "rays": int(rays.shape[0]), "ms": ms}


def update(reps: int) -> dict:
    import time

    import numpy as np

    from . import scenes
    from .wavefront import WavefrontPathTracer

    sc = scenes.large_scene()
    pt = WavefrontPathTracer({"max_depth": sc.max_depth})
    pt.set_scene(sc)
    pt.resize(64, 64)
    k = len(sc.instances) - 2   # a sphere
    xf = np.array(sc.instances[k][1], np.float32)
    out = {"workload": "update", "triangles": int(sc.world_triangles().shape[0])}
    for name, fn in (("refit_ms", lambda: pt.update_instances([k], xf[None])),
                     ("rebuild_ms", pt.rebuild_bvh)):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
        out[name] = sorted(ts)[len(ts) // 2]
    return out


def frame(res: str, views: int, nrc: bool, frames: int, scene: str = "large", seed: int = 3,
          camera_order: int = 1) -> dict:
    from . import scenes
    from .convergence import replica_views
    from .nrc import NeuralRadianceCache
    from .wavefront import WavefrontPathTracer

    w, h = (int(x) for x in res.split("x"))
    if scene == "large":
        sc = scenes.large_scene(width=w, height=h, seed=seed)
    elif scene == "cornell":
        sc = scenes.cornell_box(w, h)
    else:
        sc = scenes.volume_box(w, h)
    pt = WavefrontPathTracer({"max_depth": sc.max_depth}, seed=3)
    pt.set_scene(sc)
    pt.set_camera_order(bool(camera_order))
    if nrc:
        tris = sc.world_triangles().reshape(-1, 3)
        cache = NeuralRadianceCache(tris.min(0), tris.max(0), seed=3)
        pt.set_nrc(cache, train=True)
    pt.resize_views(replica_views(sc, views))
    out = torch.empty((pt.n_pixels, 4), device="cuda")

    def one(f):
        pt.begin_frame_views(f)
        pt.render_flat(out)

    ms = [_timed(lambda: one(f)) for f in range(1, frames + 1)]
    return {"workload": "frame", "scene": scene, "res": res, "views": views, "nrc": nrc,
            "camera_order": "tiles" if camera_order else "rows", "ms": ms,
            "device_errors": pt.device_errors()}


def batched_workload(n_views: int = 64):
    """The batched configuration: n_views views with sides log-uniform in
    [256, 1024] (view i seeded 100 + i), even views on the large scene
    (max depth 8), odd views on the volume box (max depth 16).  Returns the
    two scenes and the views as (camera, w, h, seed, scene)."""
    import math

    from . import scenes
    big = scenes.large_scene(width=64, height=64, seed=1)
    vol = scenes.volume_box(64, 64)
    views = []
    for i in range(n_views):
        rng = np.random.default_rng(100 + i)
        w = int(round(math.exp(rng.uniform(math.log(256), math.log(1024)))))
        h = int(round(math.exp(rng.uniform(math.log(256), math.log(1024)))))
        a = math.radians(rng.uniform(-10, 10))
        if i % 2 == 0:
            pos = (62.0 * math.sin(a), 22.0, -62.0 * math.cos(a))
            cam = scenes._camera(pos, (0.0, 2.0, 0.0), 45.0, w, h)
        else:
            pos = (0.5 + 1.9 * math.sin(a), 0.5, 0.5 - 1.9 * math.cos(a))
            cam = scenes._camera(pos, (0.5, 0.5, 0.0), 40.0, w, h)
        views.append((cam, w, h, 100 + i, i % 2))
    return big, vol, views


def batched(frames: int, n_views: int = 64) -> dict:
    """Eager frames of the batched configuration in one wavefront with the
    cache attached and training (default launch shapes), for launch lists."""
    from .nrc import NeuralRadianceCache
    from .wavefront import WavefrontPathTracer

    big, vol, views = batched_workload(n_views)
    pt = WavefrontPathTracer({"max_depth": 8}, seed=0)
    pt.set_scenes([big, vol])
    pt.set_scene_max_depth(1, vol.max_depth)
    pt.resize_views(views)
    lo, hi = pt.cache_box()
    pt.set_nrc(NeuralRadianceCache(lo, hi, seed=3), train=True)
    out = torch.empty((pt.n_pixels, 4), device="cuda")

    def one(f):
        pt.begin_frame_views(f)
        pt.render_flat(out)

    ms = [_timed(lambda: one(f)) for f in range(1, frames + 1)]
    return {"workload": "batched", "views": n_views, "pixels": pt.n_pixels, "ms": ms,
            "device_errors": pt.device_errors()}


def cache_curves(configs: list, res: str = "480x270", copies: int = 8, spp: int = 32768) -> list:
    """relMSE against a 65,536-spp reference of the neural-cache tracer on
    the large scene (seed 3) at 2k-32k samples per pixel, one entry per cache
    configuration (keyword arguments of NeuralRadianceCache)."""
    from . import scenes
    from .convergence import render_reference_views, time_to_error_views
    from .nrc import NeuralRadianceCache
    from .wavefront import WavefrontPathTracer

    w, h = (int(x) for x in res.split("x"))
    sc = scenes.large_scene(width=w, height=h, seed=3)
    plain = WavefrontPathTracer({"max_depth": 8}, seed=3)
    plain.set_scene(sc)
    ref = render_reference_views(plain, sc, copies, 65536 // copies)
    tris = sc.world_triangles().reshape(-1, 3)
    out = []
    for cfg in configs:
        pt = WavefrontPathTracer({"max_depth": 8}, seed=3)
        pt.set_scene(sc)
        pt.set_nrc(NeuralRadianceCache(tris.min(0), tris.max(0), seed=3, **cfg), train=True)
        r = time_to_error_views(pt, sc, ref, copies, target=0.0, max_frames=spp // copies,
                                check_every=64, max_seconds=120)
        marks = {}
        for n, e in zip(r["curve"]["timesteps"], r["curve"]["data"]):
            for m in (2048, 4096, 8192, 16384, 32768):
                if n >= m and m not in marks:
                    marks[m] = round(e, 5)
        out.append({"config": cfg, "ms_per_frame": round(r["ms_per_frame"], 3), "relmse_at_spp": marks})
        pt.close()
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("trace")
    t.add_argument("--reps", type=int, default=4)
    t.add_argument("--builder", type=int, default=2, choices=[0, 1, 2])
    t.add_argument("--levels", type=int, default=1, choices=[1, 2])
    c = sub.add_parser("cache")
    c.add_argument("--configs", default='[{"termination_spread": 0.0}]',
                   help="JSON list of cache configurations")
    c.add_argument("--res", default="480x270")
    u = sub.add_parser("update")
    u.add_argument("--reps", type=int, default=5)
    f = sub.add_parser("frame")
    f.add_argument("--scene", default="large", choices=["large", "cornell", "volume"])
    f.add_argument("--res", default="480x270")
    f.add_argument("--views", type=int, default=8)
    f.add_argument("--nrc", action="store_true")
    f.add_argument("--frames", type=int, default=3)
    f.add_argument("--seed", type=int, default=3, help="large-scene seed (the bench's 1080p frame: 1)")
    b = sub.add_parser("batched", help="eager frames of the 64-view, two-scene configuration")
    b.add_argument("--frames", type=int, default=3)
    b.add_argument("--views", type=int, default=64)
    f.add_argument("--camera-order", type=int, default=1, choices=[0, 1],
                   help="camera rays in 8x8 pixel tiles (1) or row-major (0)")
    a = ap.parse_args()
    from .build import build
    build()
    if a.cmd == "trace":
        r = trace(a.reps, a.builder, a.levels)
    elif a.cmd == "update":
        r = update(a.reps)
    elif a.cmd == "batched":
        r = batched(a.frames, a.views)
    elif a.cmd == "cache":
        r = cache_curves(json.loads(a.configs), a.res)
    else:
        r = frame(a.res, a.views, a.nrc, a.frames, a.scene, a.seed, a.camera_order)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
