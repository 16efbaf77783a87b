"""Acceleration structure: GPU LBVH -> compressed 8-wide BVH, closest-hit and
any-hit traversal (the reference's OptiX GAS/IAS and its Closest / Shadow
programs, src/core/device/optix.cpp:143-398, src/render/wavefront/device.cu:43-100).

Rays are float32 [N, 8] device tensors (origin.xyz, tmin, direction.xyz,
tmax); closest hits come back as float32 [N, 4] (t, b1, b2, triangle id bits)
with triangle id KRR_MISS = 0xFFFFFFFF for a miss.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def set_node_format(fmt: int) -> None:
    """0 = compressed 80-byte nodes (default), 1 = float 224-byte nodes."""
    check(_lib.load().krr_set_bvh_node_format(fmt), "krr_set_bvh_node_format")


def set_max_leaf(triangles: int) -> None:
    """Largest leaf (1..3 triangles) of the BVHs built from now on."""
    check(_lib.load().krr_set_bvh_max_leaf(triangles), "krr_set_bvh_max_leaf")


def set_builder(builder: int) -> None:
    """Binary tree of the BVHs built from now on: 0 radix tree on per-axis
    Morton cells, 1 PLOC clustering, 2 radix tree on cubic cells (default)."""
    check(_lib.load().krr_set_bvh_builder(builder), "krr_set_bvh_builder")


def set_collapse(mode: int) -> None:
    """How the binary tree becomes 8-wide nodes in the BVHs built from now
    on: 0 greedy (default), 1 cost-optimal (least total wide-node area)."""
    check(_lib.load().krr_set_bvh_collapse(mode), "krr_set_bvh_collapse")


def set_treelets(passes: int) -> None:
    """Treelet restructuring passes (0..3) over the binary tree of the BVHs
    built from now on (Karras and Aila 2013: seven-leaf treelets rebuilt as
    their topology of least surface area)."""
    check(_lib.load().krr_set_bvh_treelets(passes), "krr_set_bvh_treelets")


def set_full_node_leaf(triangles: int) -> None:
    """Largest leaf (1..3 triangles) among the children of a full node."""
    check(_lib.load().krr_set_bvh_full_node_leaf(triangles), "krr_set_bvh_full_node_leaf")


class Accel:
    def __init__(self, world_triangles: np.ndarray, node_format: int | None = None):
        lib = _lib.load()
        if node_format is not None:
            set_node_format(node_format)
        v = np.ascontiguousarray(world_triangles, dtype=np.float32).reshape(-1, 9)
        self._h = C.c_void_p()
        check(lib.krr_accel_create_from_triangles(v.ctypes.data, v.shape[0], C.byref(self._h),
                                                  _stream()), "krr_accel_create_from_triangles")
        self.n_triangles = v.shape[0]

    @classmethod
    def instanced(cls, geometries, instances, mask=None) -> "Accel":
        """Two-level structure: `geometries` a list of object-space triangle
        arrays (float32 [n_g, 9]); `instances` a list of (geometry index,
        float32 [3, 4] object-to-world transform); `mask` per instance (0 =
        any-hit rays pass through)."""
        lib = _lib.load()
        verts = np.ascontiguousarray(np.concatenate([np.asarray(g, np.float32).reshape(-1, 9)
                                                     for g in geometries]), dtype=np.float32)
        begin = np.zeros(len(geometries) + 1, np.int64)
        begin[1:] = np.cumsum([np.asarray(g).reshape(-1, 9).shape[0] for g in geometries])
        arr = (_lib.InstanceDesc * max(1, len(instances)))()
        for i, (g, xf) in enumerate(instances):
            arr[i].mesh = g
            arr[i].transform[:] = [float(x) for x in np.asarray(xf, np.float32).reshape(12)]
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        obj = cls.__new__(cls)
        obj._h = C.c_void_p()
        check(lib.krr_accel_create_instanced(verts.ctypes.data, begin.ctypes.data, len(geometries), arr,
                                             len(instances), None if m is None else m.ctypes.data,
                                             C.byref(obj._h), _stream()), "krr_accel_create_instanced")
        obj.n_instances = len(instances)
        obj.n_triangles = int(sum(begin[g + 1] - begin[g] for g, _ in instances))
        return obj

    def update_instances(self, transforms) -> None:
        """New object-to-world transforms, float32 [n_instances, 3, 4]."""
        x = np.ascontiguousarray(transforms, np.float32).reshape(-1, 12)
        check(_lib.load().krr_accel_update_instances(self._h, x.ctypes.data, _stream()),
              "krr_accel_update_instances")

    def instance_inverse(self) -> np.ndarray:
        out = np.empty((self.n_instances, 12), np.float32)
        check(_lib.load().krr_accel_instance_inverse(self._h, out.ctypes.data, self.n_instances),
              "krr_accel_instance_inverse")
        return out

    @classmethod
    def borrowed(cls, handle: int, n_triangles: int) -> "Accel":
        obj = cls.__new__(cls)
        obj._h = C.c_void_p(handle)
        obj.n_triangles = n_triangles
        obj._borrowed = True
        return obj

    def refit(self, world_triangles: np.ndarray) -> None:
        """New positions for the same triangles (count and order kept): the
        boxes are refitted over the existing tree."""
        v = np.ascontiguousarray(world_triangles, dtype=np.float32).reshape(-1, 9)
        check(_lib.load().krr_accel_refit_triangles(self._h, v.ctypes.data, v.shape[0], _stream()),
              "krr_accel_refit_triangles")

    def stats(self) -> dict:
        s = _lib.AccelStats()
        check(_lib.load().krr_accel_stats_get(self._h, C.byref(s)), "krr_accel_stats_get")
        d = {k: getattr(s, k) for k, _ in s._fields_ if k != "reserved"}
        d["node_format"] = s.reserved
        return d

    @staticmethod
    def _rays(rays: torch.Tensor) -> torch.Tensor:
        if not (rays.is_cuda and rays.dtype == torch.float32 and rays.dim() == 2 and
                rays.shape[1] == 8):
            raise ValueError("rays must be a CUDA float32 tensor of shape [N, 8]")
        return rays.contiguous()

    def trace_closest(self, rays: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        rays = self._rays(rays)
        n = rays.shape[0]
        if out is None:
            out = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
        check(_lib.load().krr_accel_trace_closest(self._h, rays.data_ptr(), n, out.data_ptr(),
                                                  _stream()), "krr_accel_trace_closest")
        return out

    def trace_any(self, rays: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        rays = self._rays(rays)
        n = rays.shape[0]
        if out is None:
            out = torch.empty((n,), dtype=torch.uint8, device=rays.device)
        check(_lib.load().krr_accel_trace_any(self._h, rays.data_ptr(), n, out.data_ptr(),
                                              _stream()), "krr_accel_trace_any")
        return out

    def trace_closest_host(self, rays: np.ndarray | torch.Tensor,
                           out: np.ndarray | torch.Tensor) -> None:
        """Host buffers in and out (pinned tensors are fastest)."""
        n = rays.shape[0]
        rp = rays.data_ptr() if isinstance(rays, torch.Tensor) else rays.ctypes.data
        op = out.data_ptr() if isinstance(out, torch.Tensor) else out.ctypes.data
        check(_lib.load().krr_accel_trace_closest_host(self._h, rp, n, op, _stream()),
              "krr_accel_trace_closest_host")

    def trace_stats(self, rays: torch.Tensor, any_hit: bool = False) -> tuple[int, int]:
        rays = self._rays(rays)
        counts = (C.c_ulonglong * 2)()
        check(_lib.load().krr_accel_trace_stats(self._h, rays.data_ptr(), rays.shape[0],
                                                int(any_hit), counts, _stream()),
              "krr_accel_trace_stats")
        return int(counts[0]), int(counts[1])

    def device_errors(self) -> int:
        """Error flags raised by traces since the last call (bit 0: a ray was
        cut off by the stack limit); synchronises the stream."""
        f = C.c_uint32()
        check(_lib.load().krr_accel_device_errors(self._h, C.byref(f), _stream()),
              "krr_accel_device_errors")
        return int(f.value)

    def set_stack_limit(self, entries: int) -> None:
        """Traversal stack entries a ray may use (1..48, default 48)."""
        check(_lib.load().krr_accel_set_stack_limit(self._h, entries), "krr_accel_set_stack_limit")

    def set_tuning(self, refill_below: int = 20, postpone_pct: int = 0) -> None:
        check(_lib.load().krr_accel_set_tuning(self._h, refill_below, postpone_pct), "set_tuning")

    def autotune(self, rays: torch.Tensor, repeats: int = 3) -> dict:
        """Picks the fastest traversal tuning for these rays (autotuner)."""
        rays = self._rays(rays)
        rf, pp, ms = C.c_int32(), C.c_int32(), C.c_float()
        check(_lib.load().krr_accel_autotune(self._h, rays.data_ptr(), rays.shape[0], repeats,
                                             C.byref(rf), C.byref(pp), C.byref(ms), _stream()),
              "krr_accel_autotune")
        return {"refill_below": rf.value, "postpone_pct": pp.value, "ms": ms.value}

    def set_mask(self, mask: np.ndarray | None) -> None:
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        check(_lib.load().krr_accel_set_mask(self._h, None if m is None else m.ctypes.data),
              "krr_accel_set_mask")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value and not getattr(self, "_borrowed", False):
            _lib.load().krr_accel_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
