"""Image passes after the path tracer: FP64 accumulation and relMSE against a
reference image, in the manner of the reference's AccumulatePass ("double"
precision, src/render/passes/accumulate/accumulate.cu:30-79) and
ErrorMeasurePass (src/render/passes/errormeasure/errormeasure.cpp:17-57,
metrics.cu:64-128), which logs a curve {timesteps, timepoints, data}; and
the ToneMappingPass (src/render/passes/tonemapping/tonemapping.cu:60-88).
"""
from __future__ import annotations

import ctypes as C
import time

import torch

from . import _lib
from ._lib import check

RELMSE, MSE = 0, 1


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class Accumulator:
    """FP64 running sum of float4 RGBA frames (device resident)."""

    def __init__(self, width: int, height: int):
        self.n = width * height
        self.sum = torch.zeros((self.n, 3), dtype=torch.float64, device="cuda")
        self.frames = 0

    def add(self, rgba: torch.Tensor):
        check(_lib.load().krr_accumulate_f64(rgba.data_ptr(), self.sum.data_ptr(), self.n,
                                             _stream()), "krr_accumulate_f64")
        self.frames += 1

    MAGIC = b"KRRACC01"

    def save(self, path) -> None:
        """Checkpoint of the FP64 running sum and its frame count (a header
        of magic, pixel count and frames, then n x 3 float64), so that a
        convergence run can resume."""
        import numpy as np
        torch.cuda.synchronize()
        with open(path, "wb") as f:
            f.write(self.MAGIC)
            f.write(np.array([self.n, self.frames], np.int64).tobytes())
            f.write(self.sum.cpu().numpy().astype(np.float64).tobytes())

    def load(self, path) -> None:
        import numpy as np
        with open(path, "rb") as f:
            if f.read(8) != self.MAGIC:
                raise ValueError(f"{path} is not an accumulation checkpoint")
            n, frames = np.frombuffer(f.read(16), np.int64)
            if n != self.n:
                raise ValueError(f"{path} holds {n} pixels, this accumulator {self.n}")
            data = np.frombuffer(f.read(int(n) * 24), np.float64)
            if data.size != 3 * n:
                raise ValueError(f"{path} is truncated")
        self.sum.copy_(torch.from_numpy(data.reshape(-1, 3).copy()))
        self.frames = int(frames)

    def image(self) -> torch.Tensor:
        """float32 [n, 4] mean image."""
        out = torch.ones((self.n, 4), dtype=torch.float32, device="cuda")
        out[:, :3] = (self.sum / max(self.frames, 1)).float()
        return out

    def error(self, ref_rgba: torch.Tensor, metric: int = RELMSE) -> float:
        v = C.c_double()
        check(_lib.load().krr_image_error(self.sum.data_ptr(), 1.0 / max(self.frames, 1),
                                          ref_rgba.data_ptr(), self.n, metric, C.byref(v),
                                          _stream()), "krr_image_error")
        return v.value


TONEMAP_OPERATORS = ("linear", "reinhard", "aces", "uncharted2", "hejihable")


def tonemap(rgba: torch.Tensor, operator: str = "linear", exposure: float = 1.0, gamma: bool = True,
            out: torch.Tensor | None = None) -> torch.Tensor:
    """The reference's ToneMappingPass with its JSON parameters ("operator",
    "exposure", "gamma"; tonemapping.h:40-51) on a float4 RGBA image."""
    if not (rgba.is_cuda and rgba.dtype == torch.float32 and rgba.shape[-1] == 4):
        raise ValueError("rgba must be a CUDA float32 tensor with 4 channels last")
    rgba = rgba.contiguous()
    out = torch.empty_like(rgba) if out is None else out
    check(_lib.load().krr_tonemap(rgba.data_ptr(), out.data_ptr(), rgba.numel() // 4,
                                  TONEMAP_OPERATORS.index(operator), float(exposure), int(bool(gamma)),
                                  _stream()), "krr_tonemap")
    return out


def replica_views(scene, copies: int, seed_base: int = 0) -> list:
    """`copies` views of the scene's camera whose seeds are 2^24 apart, so
    that frame f of view k (sample index f + seed) never repeats another
    view's sample index while f < 2^24."""
    return [(scene.camera, scene.width, scene.height, seed_base + (k << 24)) for k in range(copies)]


def _add_views(acc: "Accumulator", flat: torch.Tensor, copies: int):
    n = acc.n
    for k in range(copies):
        acc.add(flat[k * n:(k + 1) * n])


def render_reference_views(pt, scene, copies: int, frames: int,
                           first_frame: int = 1 << 22) -> torch.Tensor:
    """FP64 mean of frames x copies samples per pixel: `copies` replicas of
    the camera traced together in each launch (a captured frame graph
    replayed `frames` times).  Frame indices start at `first_frame`, away
    from those of a measured run.  Returns float32 [n, 4]."""
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        pt.resize_views(replica_views(scene, copies))
        acc = Accumulator(scene.width, scene.height)
        out = torch.empty((copies * acc.n, 4), dtype=torch.float32, device="cuda")
        pt.begin_frame_views(first_frame)
        pt.render_flat(out)
        _add_views(acc, out, copies)
        pt.capture_frame(out)
        for f in range(1, frames):
            pt.launch_frame(first_frame + f)
            _add_views(acc, out, copies)
        img = acc.image()
    stream.synchronize()
    return img


def time_to_error_views(pt, scene, ref_rgba: torch.Tensor, copies: int, target: float = 0.01,
                        max_frames: int = 4096, check_every: int = 16, metric: int = RELMSE,
                        max_seconds: float | None = None) -> dict:
    """time_to_error with `copies` replicas of the camera per launch (so each
    frame adds `copies` samples per pixel) and frames replayed from a
    captured graph.  Device time of rendering and accumulation counts;
    error evaluation does not.  Curve timesteps are samples per pixel."""
    stream = torch.cuda.Stream()
    curve = {"timesteps": [], "timepoints": [], "data": []}
    reached = None
    with torch.cuda.stream(stream):
        pt.resize_views(replica_views(scene, copies))
        acc = Accumulator(scene.width, scene.height)
        out = torch.empty((copies * acc.n, 4), dtype=torch.float32, device="cuda")
        t_ms = 0.0
        pending = []
        for f in range(1, max_frames + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if f == 1:
                pt.begin_frame_views(1)
                pt.render_flat(out)
            else:
                pt.launch_frame(f)
            _add_views(acc, out, copies)
            e1.record(stream)
            pending.append((e0, e1))
            if f == 1:
                stream.synchronize()
                pt.capture_frame(out)
            if f % check_every == 0 or f == max_frames:
                stream.synchronize()
                t_ms += sum(a.elapsed_time(b) for a, b in pending)
                pending = []
                err = acc.error(ref_rgba, metric)
                curve["timesteps"].append(acc.frames)
                curve["timepoints"].append(t_ms / 1e3)
                curve["data"].append(err)
                if err <= target:
                    reached = t_ms / 1e3
                    break
                if max_seconds is not None and t_ms / 1e3 >= max_seconds:
                    break
    stream.synchronize()
    return {"seconds": reached, "spp": acc.frames, "frames": acc.frames // copies,
            "curve": curve, "ms_per_frame": t_ms / max(1, acc.frames // copies),
            "final_error": curve["data"][-1] if curve["data"] else None}


def render_reference(pt, scene, frames: int, first_frame: int = 1_000_000) -> torch.Tensor:
    """Mean of `frames` 1-spp frames accumulated in FP64 (float32 [n, 4])."""
    acc = Accumulator(scene.width, scene.height)
    out = torch.empty((scene.height, scene.width, 4), dtype=torch.float32, device="cuda")
    for f in range(frames):
        pt.begin_frame(first_frame + f, scene.camera)
        pt.render(out)
        acc.add(out)
    return acc.image()


def time_to_error(pt, scene, ref_rgba: torch.Tensor, target: float = 0.01, max_frames: int = 4096,
                  check_every: int = 4, metric: int = RELMSE, on_frame=None) -> dict:
    """Renders 1-spp frames until the running mean reaches `target` error.

    Only the device time of rendering (and of on_frame, e.g. cache training)
    counts; error evaluation is excluded.  Returns the curve
    {timesteps, timepoints, data} and the time at which the target was met
    (None if it was not within max_frames)."""
    acc = Accumulator(scene.width, scene.height)
    out = torch.empty((scene.height, scene.width, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    t_ms = 0.0
    curve = {"timesteps": [], "timepoints": [], "data": []}
    reached = None
    for f in range(1, max_frames + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pt.begin_frame(f, scene.camera)
        pt.render(out)
        if on_frame is not None:
            on_frame(f, out)
        acc.add(out)
        e1.record(stream)
        e1.synchronize()
        t_ms += e0.elapsed_time(e1)
        if f % check_every == 0 or f == max_frames:
            err = acc.error(ref_rgba, metric)
            curve["timesteps"].append(f)
            curve["timepoints"].append(t_ms / 1e3)
            curve["data"].append(err)
            if err <= target:
                reached = t_ms / 1e3
                break
    return {"seconds": reached, "frames": acc.frames, "curve": curve,
            "final_error": curve["data"][-1] if curve["data"] else None}
