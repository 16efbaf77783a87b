"""ctypes loader of oracle/liboracle.so (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
_lib = None


def build(force: bool = False) -> Path:
    deps = list(HERE.glob("*.cpp")) + list(HERE.glob("*.h"))
    if force or not LIB.exists() or any(p.stat().st_mtime > LIB.stat().st_mtime for p in deps):
        jobs = str(min(16, os.cpu_count() or 4))
        subprocess.run(["make", "-s", "-j", jobs, "-C", str(HERE)], check=True)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        P, I64 = C.c_void_p, C.c_int64
        sig = {
            "oracle_bvh_build": (C.c_int, [P, I64, C.c_int, C.POINTER(P)]),
            "oracle_bvh_free": (None, [P]),
            "oracle_bvh_set_mask": (None, [P, P]),
            "oracle_trace_closest": (C.c_int, [P, P, I64, P, C.c_int]),
            "oracle_trace_any": (C.c_int, [P, P, I64, P, C.c_int]),
            "oracle_trace_closest_brute": (C.c_int, [P, I64, P, I64, P]),
            "oracle_pcg_floats": (None, [C.c_uint32, C.c_uint32, C.c_uint32, I64, C.c_int, P]),
            "oracle_pcg_u32": (None, [C.c_uint64, C.c_uint64, C.c_int, P]),
            "oracle_interleave_32bit": (C.c_uint32, [C.c_uint32, C.c_uint32]),
            "oracle_fr_dielectric": (C.c_float, [C.c_float, C.c_float]),
            "oracle_bsdf_eval": (None, [P, P, P, I64, P]),
            "oracle_bsdf_sample": (None, [P, P, P, I64, P]),
            "oracle_hg_p": (C.c_float, [C.c_float, P, P]),
            "oracle_hg_sample": (None, [C.c_float, P, P, I64, P]),
            "oracle_light_sample": (C.c_int, [P, C.c_int32, P, P, I64, P]),
            "oracle_light_count": (C.c_int32, [P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def threads() -> int:
    return max(1, os.cpu_count() or 1)


class Bvh:
    def __init__(self, tris: np.ndarray):
        self.tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
        self._h = C.c_void_p()
        load().oracle_bvh_build(self.tris.ctypes.data, self.tris.shape[0], threads(),
                                C.byref(self._h))

    def set_mask(self, mask):
        self._mask = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        load().oracle_bvh_set_mask(self._h, None if self._mask is None else self._mask.ctypes.data)

    def closest(self, rays: np.ndarray, nthreads: int | None = None) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.empty((rays.shape[0], 4), np.float32)
        load().oracle_trace_closest(self._h, rays.ctypes.data, rays.shape[0], out.ctypes.data,
                                    nthreads or threads())
        return out

    def any(self, rays: np.ndarray, nthreads: int | None = None) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.empty((rays.shape[0],), np.uint8)
        load().oracle_trace_any(self._h, rays.ctypes.data, rays.shape[0], out.ctypes.data,
                                nthreads or threads())
        return out

    def __del__(self):
        try:
            if self._h:
                load().oracle_bvh_free(self._h)
        except Exception:
            pass


def closest_brute(tris: np.ndarray, rays: np.ndarray) -> np.ndarray:
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    out = np.empty((rays.shape[0], 4), np.float32)
    load().oracle_trace_closest_brute(tris.ctypes.data, tris.shape[0], rays.ctypes.data,
                                      rays.shape[0], out.ctypes.data)
    return out


def trace_instanced(geometries, instances, inverse, rays, mask=None, any_hit=False):
    """Two-level closest (or any) hits: geometries as float32 [n_g, 9]
    object-space triangles, instances as (geometry, transform) pairs whose
    world-to-object matrices are `inverse` [n_inst, 12] (the ones the GPU
    structure uses), global ids instance-major."""
    lib = load()
    fn = lib.oracle_trace_instanced
    fn.restype = C.c_int
    P, I64 = C.c_void_p, C.c_int64
    fn.argtypes = [P, P, C.c_int, P, P, P, P, C.c_int, P, I64, P, P, C.c_int]
    verts = np.ascontiguousarray(np.concatenate([np.asarray(g, np.float32).reshape(-1, 9)
                                                 for g in geometries]), dtype=np.float32)
    counts = [np.asarray(g).reshape(-1, 9).shape[0] for g in geometries]
    begin = np.zeros(len(geometries) + 1, np.int64)
    begin[1:] = np.cumsum(counts)
    geom = np.array([g for g, _ in instances], np.int32)
    first = np.zeros(len(instances), np.int64)
    first[1:] = np.cumsum([counts[g] for g in geom])[:-1]
    inv = np.ascontiguousarray(inverse, np.float32).reshape(-1, 12)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    hits = np.empty((rays.shape[0], 4), np.float32)
    occ = np.empty(rays.shape[0], np.uint8)
    fn(verts.ctypes.data, begin.ctypes.data, len(geometries), geom.ctypes.data, inv.ctypes.data,
       first.ctypes.data, None if m is None else m.ctypes.data, len(instances), rays.ctypes.data,
       rays.shape[0], None if any_hit else hits.ctypes.data, occ.ctypes.data if any_hit else None,
       threads())
    return occ if any_hit else hits


def pcg_floats(px: int, py: int, sample_index: int, advance: int, count: int) -> np.ndarray:
    out = np.empty(count, np.float32)
    load().oracle_pcg_floats(px, py, sample_index, advance, count, out.ctypes.data)
    return out


def pcg_u32(initstate: int, initseq: int, count: int) -> np.ndarray:
    out = np.empty(count, np.uint32)
    load().oracle_pcg_u32(initstate, initseq, count, out.ctypes.data)
    return out


MAT_DIFFUSE, MAT_DIELECTRIC, MAT_CONDUCTOR = 1, 2, 3


def material(kind: int, color=(0.8, 0.8, 0.8), roughness: float = 0.5, spec_trans: float = 0.0,
              ior: float = 1.5, anisotropic: float = 0.0) -> np.ndarray:
    return np.array([kind, *color, roughness, spec_trans, ior, anisotropic], np.float32)


def fr_dielectric(cos_i: float, eta: float) -> float:
    return float(load().oracle_fr_dielectric(cos_i, eta))


def bsdf_eval(material: np.ndarray, wo: np.ndarray, wi: np.ndarray) -> np.ndarray:
    """f (rgb) and pdf [n, 4] of direction pairs in the local shading frame."""
    wo = np.ascontiguousarray(np.broadcast_to(wo, np.shape(wi)), np.float32).reshape(-1, 3)
    wi = np.ascontiguousarray(wi, np.float32).reshape(-1, 3)
    out = np.empty((wi.shape[0], 4), np.float32)
    load().oracle_bsdf_eval(material.ctypes.data, wo.ctypes.data, wi.ctypes.data, wi.shape[0],
                            out.ctypes.data)
    return out


def bsdf_sample(material: np.ndarray, wo, u: np.ndarray) -> np.ndarray:
    """Samples [n, 8] (f rgb, wi xyz, pdf, flags) for one wo, row i drawing u[i, 0..2]."""
    wo = np.ascontiguousarray(wo, np.float32)
    u = np.ascontiguousarray(u, np.float32).reshape(-1, 3)
    out = np.empty((u.shape[0], 8), np.float32)
    load().oracle_bsdf_sample(material.ctypes.data, wo.ctypes.data, u.ctypes.data, u.shape[0],
                              out.ctypes.data)
    return out


def hg_p(g: float, wo, wi) -> float:
    wo = np.ascontiguousarray(wo, np.float32)
    wi = np.ascontiguousarray(wi, np.float32)
    return float(load().oracle_hg_p(g, wo.ctypes.data, wi.ctypes.data))


def hg_sample(g: float, wo, u: np.ndarray) -> np.ndarray:
    """Samples [n, 4] (wi xyz, pdf) of the HG phase function around wo."""
    wo = np.ascontiguousarray(wo, np.float32)
    u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
    out = np.empty((u.shape[0], 4), np.float32)
    load().oracle_hg_sample(g, wo.ctypes.data, u.ctypes.data, u.shape[0], out.ctypes.data)
    return out


class PathTracer:
    """CPU restatement of the wavefront path tracer (oracle/pathtracer.cpp)."""

    def __init__(self, scene):
        from kiraray_gb300 import _lib as L
        lib = load()
        lib.oracle_pt_create.restype = C.c_int
        lib.oracle_pt_create.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        lib.oracle_pt_free.argtypes = [C.c_void_p]
        lib.oracle_pt_render.restype = C.c_int
        lib.oracle_pt_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                         C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                         C.c_int]
        self._L = L
        self.scene = scene
        self._desc, self._keep = scene.desc()
        self._h = C.c_void_p()
        lib.oracle_pt_create(C.byref(self._desc), threads(), C.byref(self._h))

    def render(self, params: dict, frame_index: int, px_begin: int = 0, px_end: int | None = None,
               spp: int = 1, seed: int = 0, camera=None):
        L = self._L
        p = L.WfParams()
        p.nee, p.enable_medium, p.max_depth, p.rr = 1, 1, 10, 0.8
        p.enable_clamp, p.clamp_max, p.spp, p.seed = 0, 1e3, spp, seed
        for k, v in params.items():
            setattr(p, k, type(getattr(p, k))(v))
        sc = self.scene
        cam = (camera or sc.camera).desc()
        n_total = sc.width * sc.height
        px_end = n_total if px_end is None else px_end
        n = px_end - px_begin
        out_L = np.zeros((n, 3), np.float32)
        out_px = np.zeros((n, 3), np.float32)
        load().oracle_pt_render(self._h, C.byref(p), C.byref(cam), sc.width, sc.height,
                                frame_index, px_begin, px_end, out_L.ctypes.data,
                                out_px.ctypes.data, threads())
        return out_L, out_px

    def light_count(self) -> int:
        return int(load().oracle_light_count(self._h))

    def light_sample(self, light: int, cp, u: np.ndarray) -> np.ndarray:
        """[n, 8]: p xyz, L rgb, solid-angle pdf, hit-side pdf of the same point."""
        cp = np.ascontiguousarray(cp, np.float32)
        u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
        out = np.empty((u.shape[0], 8), np.float32)
        if load().oracle_light_sample(self._h, light, cp.ctypes.data, u.ctypes.data, u.shape[0],
                                      out.ctypes.data):
            raise IndexError(light)
        return out

    def __del__(self):
        try:
            load().oracle_pt_free(self._h)
        except Exception:
            pass
