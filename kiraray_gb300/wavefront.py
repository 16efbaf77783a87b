"""Host-side mirror of the reference's WavefrontPathTracer render pass
(src/render/wavefront/integrator.h:24-104) over the C ABI.

    pt = WavefrontPathTracer({"max_depth": 5, "rr": 0.8, "nee": True})
    pt.set_scene(scene)          # RenderPass::setScene
    pt.resize(w, h)              # RenderPass::resize
    pt.begin_frame(1, camera)    # RenderPass::beginFrame (frame index is 1-based)
    img = pt.render()            # RenderPass::render -> float32 [H, W, 4] on the GPU

Stage methods keep the reference's names for PPG-style subclasses.  Device
buffers are torch CUDA tensors; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check

PARAM_NAMES = ("nee", "enable_medium", "max_depth", "rr", "enable_clamp", "clamp_max")


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class _DeviceArray:
    """float32 device memory owned by the pass, seen through the CUDA array
    interface (no copy)."""

    def __init__(self, ptr: int, shape: tuple):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": "<f4", "data": (ptr, False),
                                         "version": 3, "strides": None}


class WavefrontPathTracer:
    def __init__(self, params: dict | None = None, spp: int = 1, seed: int = 0):
        self.lib = _lib.load()
        self.params = _lib.WfParams()
        self.lib.krr_wf_params_default(C.byref(self.params))
        self.params.spp = spp
        self.params.seed = seed
        self._apply(params or {})
        self._h = C.c_void_p()
        check(self.lib.krr_wf_create(C.byref(self.params), C.byref(self._h)), "krr_wf_create")
        self.width = self.height = 0
        self._keep = None
        self.scene = None

    @classmethod
    def from_json(cls, params_json: str) -> "WavefrontPathTracer":
        """The pass created from its JSON parameters through the C ABI
        (krr_wf_create_json: the reference's from_json keys and defaults)."""
        obj = cls.__new__(cls)
        obj.lib = _lib.load()
        obj._h = C.c_void_p()
        check(obj.lib.krr_wf_create_json(params_json.encode(), C.byref(obj._h)), "krr_wf_create_json")
        obj.params = _lib.WfParams()
        check(obj.lib.krr_wf_get_params(obj._h, C.byref(obj.params)), "krr_wf_get_params")
        obj.width = obj.height = 0
        obj._keep = None
        obj.scene = None
        return obj

    def set_params_json(self, params_json: str):
        check(self.lib.krr_wf_set_params_json(self._h, params_json.encode()), "krr_wf_set_params_json")
        check(self.lib.krr_wf_get_params(self._h, C.byref(self.params)), "krr_wf_get_params")

    # from_json, integrator.h:94-103
    def _apply(self, params: dict):
        for k, v in params.items():
            if k not in PARAM_NAMES + ("spp", "seed", "independent_samples"):
                raise KeyError(f"unknown parameter {k!r}")
            setattr(self.params, k, type(getattr(self.params, k))(v))

    def set_params(self, params: dict):
        self._apply(params)
        check(self.lib.krr_wf_set_params(self._h, C.byref(self.params)), "krr_wf_set_params")

    def get_name(self) -> str:
        return "WavefrontPathTracer"

    def set_scene(self, scene):
        desc, keep = scene.desc()
        check(self.lib.krr_wf_set_scene(self._h, C.byref(desc), _stream()), "krr_wf_set_scene")
        self._keep = (desc, keep)
        self.scene = scene

    def update_instances(self, indices, transforms) -> None:
        """New 3x4 transforms (float32 [n, 3, 4] or [n, 12]) for the given
        instances; refits the BVH's boxes over its tree (Scene::update with
        animation).  A captured frame stays valid."""
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int32))
        xf = np.ascontiguousarray(np.asarray(transforms, dtype=np.float32).reshape(-1, 12))
        if xf.shape[0] != idx.shape[0]:
            raise ValueError("one transform per instance index")
        check(self.lib.krr_wf_update_instances(self._h, int(idx.shape[0]), idx.ctypes.data,
                                               xf.ctypes.data, _stream()), "update_instances")

    def rebuild_bvh(self) -> None:
        """Full BVH build over the current instance transforms."""
        check(self.lib.krr_wf_rebuild_bvh(self._h, _stream()), "rebuild_bvh")

    def set_nrc(self, cache, train: bool = True):
        """Attaches a NeuralRadianceCache (None detaches: the plain tracer)."""
        self._nrc = cache
        check(self.lib.krr_wf_set_nrc(self._h, cache._h if cache is not None else None,
                                      int(bool(train))), "krr_wf_set_nrc")

    def resize(self, width: int, height: int):
        check(self.lib.krr_wf_resize(self._h, width, height), "krr_wf_resize")
        self.width, self.height = width, height
        self.n_pixels = width * height
        self._views = None

    @staticmethod
    def _view_array(views):
        """(camera, width, height, seed[, scene]) tuples -> krr_view array."""
        arr = (_lib.ViewDesc * len(views))()
        for i, v in enumerate(views):
            cam, w, h, seed = v[:4]
            arr[i].camera = cam.desc()
            arr[i].width, arr[i].height, arr[i].seed = w, h, seed
            arr[i].scene = v[4] if len(v) > 4 else 0
        return arr

    def resize_views(self, views):
        """Batched views: list of (camera, width, height, seed[, scene])."""
        arr = self._view_array(views)
        check(self.lib.krr_wf_resize_views(self._h, arr, len(views)), "krr_wf_resize_views")
        self._views = arr
        self.width = self.height = 0
        self.n_pixels = sum(v[1] * v[2] for v in views)

    def set_scenes(self, scenes):
        """Several scenes in one wavefront; views name theirs by index."""
        descs = [sc.desc() for sc in scenes]
        arr = (_lib.SceneDesc * len(scenes))(*[d for d, _ in descs])
        check(self.lib.krr_wf_set_scenes(self._h, arr, len(scenes), _stream()), "krr_wf_set_scenes")
        self._keep = (descs, arr)
        self.scene = scenes[0]
        self.scenes = list(scenes)

    def set_launch(self, block: int = 256, blocks_per_sm: int = 8, wave: int = 0) -> None:
        """Stage-kernel launch shapes and the queue capacity (wave 0: every
        pixel at once)."""
        check(self.lib.krr_wf_set_launch(self._h, block, blocks_per_sm, wave), "krr_wf_set_launch")

    def launch(self) -> dict:
        b, bps, w, cap = C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64()
        check(self.lib.krr_wf_get_launch(self._h, C.byref(b), C.byref(bps), C.byref(w), C.byref(cap)),
              "krr_wf_get_launch")
        return {"block": b.value, "blocks_per_sm": bps.value, "wave": w.value,
                "queue_capacity": cap.value}

    def autotune(self, out: torch.Tensor, frames: int = 3) -> dict:
        """Times frames for each candidate launch shape / queue capacity and
        keeps the fastest (krr_wf_autotune)."""
        t = _lib.WfTuning()
        check(self.lib.krr_wf_autotune(self._h, out.data_ptr(), frames, C.byref(t), _stream()),
              "krr_wf_autotune")
        return {k: getattr(t, k) for k, _ in t._fields_ if k != "reserved"}

    def set_megakernel_reorder(self, reorder: bool) -> None:
        """Megakernel variant: regroup a block's paths by hit class after
        each closest hit (default) or keep one path per thread."""
        check(self.lib.krr_wf_set_megakernel_reorder(self._h, int(bool(reorder))),
              "krr_wf_set_megakernel_reorder")

    def set_media_order(self, order: bool) -> None:
        """Medium tracking items taken by estimated optical depth (True) or
        in queue order (False, default)."""
        check(self.lib.krr_wf_set_media_order(self._h, int(bool(order))), "krr_wf_set_media_order")

    def set_profiling(self, on: bool) -> None:
        """Per-stage device timers (the reference's PROFILE events), off by default."""
        check(self.lib.krr_wf_set_profiling(self._h, int(bool(on))), "krr_wf_set_profiling")

    def profile(self) -> dict:
        """Stage -> (calls, device ms) since the last call; waits for the timed work."""
        buf = (_lib.StageTime * 32)()
        n = C.c_int32()
        check(self.lib.krr_wf_profile_read(self._h, buf, 32, C.byref(n)), "krr_wf_profile_read")
        return {buf[i].name.decode(): (int(buf[i].calls), float(buf[i].ms))
                for i in range(min(n.value, 32))}

    def set_camera_order(self, tiled: bool) -> None:
        """Camera rays queued in 8x8 pixel tiles (True, default) or row-major."""
        check(self.lib.krr_wf_set_camera_order(self._h, int(bool(tiled))), "krr_wf_set_camera_order")

    def set_accel_levels(self, levels: int) -> None:
        """1: flattened instances (default), 2: two-level structure."""
        check(self.lib.krr_wf_set_accel_levels(self._h, levels), "krr_wf_set_accel_levels")

    def set_scene_max_depth(self, scene: int, max_depth: int) -> None:
        """Path depth of one scene of the pass (-1: the pass's)."""
        check(self.lib.krr_wf_set_scene_max_depth(self._h, scene, max_depth),
              "krr_wf_set_scene_max_depth")

    def cache_box(self):
        lo, hi = (C.c_float * 3)(), (C.c_float * 3)()
        check(self.lib.krr_wf_cache_box(self._h, lo, hi), "krr_wf_cache_box")
        return tuple(lo), tuple(hi)

    def begin_frame_views(self, frame_index: int, views=None):
        if views is not None:
            self._views = self._view_array(views)
        check(self.lib.krr_wf_begin_frame_views(self._h, frame_index, self._views,
                                                len(self._views), _stream()),
              "krr_wf_begin_frame_views")

    def render_flat(self, out: torch.Tensor | None = None) -> torch.Tensor:
        """render() for a batched layout: float32 [total pixels, 4]."""
        if out is None:
            out = torch.empty((self.n_pixels, 4), dtype=torch.float32, device="cuda")
        check(self.lib.krr_wf_render(self._h, out.data_ptr(), _stream()), "krr_wf_render")
        return out

    def capture_frame(self, out: torch.Tensor):
        """Captures beginFrame + render into a CUDA graph writing `out`."""
        check(self.lib.krr_wf_capture_frame(self._h, out.data_ptr(), _stream()),
              "krr_wf_capture_frame")

    def launch_frame(self, frame_index: int):
        views = getattr(self, "_views", None)
        check(self.lib.krr_wf_launch_frame(self._h, frame_index, views,
                                           len(views) if views is not None else 0, _stream()),
              "krr_wf_launch_frame")

    def begin_frame(self, frame_index: int, camera):
        self._cam = camera.desc()
        check(self.lib.krr_wf_begin_frame(self._h, frame_index, C.byref(self._cam), _stream()),
              "krr_wf_begin_frame")

    def render(self, out: torch.Tensor | None = None) -> torch.Tensor:
        if out is None:
            out = torch.empty((self.height, self.width, 4), dtype=torch.float32, device="cuda")
        check(self.lib.krr_wf_render(self._h, out.data_ptr(), _stream()), "krr_wf_render")
        return out

    def render_megakernel(self, out: torch.Tensor | None = None) -> torch.Tensor:
        """The same frame as render() from one persistent kernel (surfaces only)."""
        if out is None:
            out = torch.empty((self.height, self.width, 4), dtype=torch.float32, device="cuda")
        check(self.lib.krr_wf_render_megakernel(self._h, out.data_ptr(), _stream()),
              "krr_wf_render_megakernel")
        return out

    # stage methods (integrator.cpp:50-179)
    def generate_camera_rays(self):
        check(self.lib.krr_wf_generate_camera_rays(self._h, _stream()), "generate_camera_rays")

    def reset_queues(self, depth: int):
        check(self.lib.krr_wf_reset_queues(self._h, depth, _stream()), "reset_queues")

    def trace_closest(self, depth: int):
        check(self.lib.krr_wf_trace_closest(self._h, depth, _stream()), "trace_closest")

    def handle_hit(self):
        check(self.lib.krr_wf_handle_hit(self._h, _stream()), "handle_hit")

    def handle_miss(self):
        check(self.lib.krr_wf_handle_miss(self._h, _stream()), "handle_miss")

    def generate_scatter_rays(self, depth: int):
        check(self.lib.krr_wf_generate_scatter_rays(self._h, depth, _stream()), "scatter")

    def trace_shadow(self):
        check(self.lib.krr_wf_trace_shadow(self._h, _stream()), "trace_shadow")

    def sample_medium_interaction(self, depth: int):
        check(self.lib.krr_wf_sample_medium_interaction(self._h, depth, _stream()), "medium")

    def sample_medium_scattering(self, depth: int):
        check(self.lib.krr_wf_sample_medium_scattering(self._h, depth, _stream()), "medium")

    def queue_size(self, queue: int) -> int:
        v = C.c_int32()
        check(self.lib.krr_wf_queue_size(self._h, queue, C.byref(v), _stream()), "queue_size")
        return v.value

    def queue_items(self, queue: int) -> torch.Tensor:
        """Copy of a queue's live items: float32 [count, channels, 4]."""
        base, ch, cap = C.c_void_p(), C.c_int32(), C.c_int32()
        check(self.lib.krr_wf_queue_view(self._h, queue, C.byref(base), C.byref(ch), C.byref(cap)),
              "queue_view")
        n = self.queue_size(queue)
        planes = torch.as_tensor(_DeviceArray(base.value, (ch.value, cap.value, 4)), device="cuda")
        return planes[:, :n, :].permute(1, 0, 2).contiguous()

    def radiance(self) -> torch.Tensor:
        """Per-pixel L (the reference's PixelState::L) as float32 [pixels, 4]."""
        out = torch.empty((self.n_pixels, 4), dtype=torch.float32, device="cuda")
        check(self.lib.krr_wf_read_radiance(self._h, out.data_ptr(), _stream()), "read_radiance")
        return out

    def set_loop_limits(self, max_null_collisions: int = 1 << 20,
                        max_interface_crossings: int = 64) -> None:
        """Bounds of the medium tracking loops; a walk that runs out raises
        the loop-limit flag (bit 2 of device_errors) and ends."""
        check(self.lib.krr_wf_set_loop_limits(self._h, max_null_collisions,
                                              max_interface_crossings), "set_loop_limits")

    def device_errors(self) -> int:
        v = C.c_uint32()
        check(self.lib.krr_wf_device_errors(self._h, C.byref(v), _stream()), "device_errors")
        return v.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.krr_wf_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FrameGroup:
    """Several passes rendered as one CUDA graph with one branch per pass
    (e.g. two scenes with their batched views); see krr_wf_group_*."""

    def __init__(self, passes, outs):
        if len(passes) != len(outs):
            raise ValueError("one output per pass")
        self.lib = _lib.load()
        self.passes, self.outs = list(passes), list(outs)
        n = len(self.passes)
        hp = (C.c_void_p * n)(*[p._h.value for p in self.passes])
        ho = (C.c_void_p * n)(*[o.data_ptr() for o in self.outs])
        self._h = C.c_void_p()
        check(self.lib.krr_wf_group_create(hp, ho, n, C.byref(self._h)), "krr_wf_group_create")

    def capture(self):
        check(self.lib.krr_wf_group_capture(self._h, _stream()), "krr_wf_group_capture")

    def launch(self, frame_index: int):
        check(self.lib.krr_wf_group_launch(self._h, frame_index, _stream()), "krr_wf_group_launch")

    def close(self):
        if self._h:
            self.lib.krr_wf_group_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
