"""Heterogeneous and homogeneous media on the GPU against the CPU restatement
(per pixel, same tolerance as tests/test_wavefront_gpu.py)."""
import numpy as np
import pytest

from kiraray_gb300 import scenes
from kiraray_gb300.wavefront import WavefrontPathTracer
from oracle import pyoracle as O
from tests.test_wavefront_gpu import compare, gpu_frame

pytestmark = pytest.mark.gpu


def _run(sc, params, frame):
    pt = WavefrontPathTracer(params)
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    L, img = gpu_frame(pt, sc, frame)
    assert pt.device_errors() == 0
    oL, _ = O.PathTracer(sc).render(params, frame)
    return L[:, :3], oL, img


@pytest.mark.parametrize("frame", [1, 4])
def test_volume_box_delta_and_ratio_tracking(krr_lib, cuda, frame):
    sc = scenes.volume_box(96, 96, max_depth=16, grid=64)
    L, oL, img = _run(sc, {"max_depth": 16}, frame)
    compare(L, oL, f"volume frame {frame}")
    assert np.isfinite(img).all()


def test_homogeneous_medium(krr_lib, cuda):
    sc = scenes.volume_box(80, 80, max_depth=10, grid=16)
    sc.media[0] = scenes.Medium(None, sc.media[0].bounds_min, sc.media[0].bounds_max,
                                sigma_t=(3.0, 2.0, 1.0), albedo=(0.8, 0.85, 0.9), g=-0.4)
    L, oL, _ = _run(sc, {"max_depth": 10}, 2)
    compare(L, oL, "homogeneous medium")


def test_medium_disabled_ignores_media(krr_lib, cuda):
    sc = scenes.volume_box(64, 64, max_depth=6, grid=32)
    L, oL, _ = _run(sc, {"max_depth": 6, "enable_medium": False}, 1)
    compare(L, oL, "media disabled")
    # with media off the null box only relays rays (each crossing still uses
    # one bounce of the loop, as in the reference): no pixel goes black
    assert (L.sum(1) > 0).mean() > 0.4


def test_loop_limits_raise_the_flag_and_end_the_walk(krr_lib, cuda):
    """A null-collision bound of 1 ends the tracking walks early and raises
    the loop-limit flag (bit 2); the defaults raise nothing and match the
    oracle again."""
    sc = scenes.volume_box(64, 64, max_depth=8, grid=32)
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    pt.set_loop_limits(1, 64)
    L, img = gpu_frame(pt, sc, 1)
    assert pt.device_errors() & 4
    assert np.isfinite(img).all()
    pt.set_loop_limits(1 << 20, 1)
    gpu_frame(pt, sc, 1)
    assert pt.device_errors() & 4   # shadow rays cross the box's two null interfaces
    pt.set_loop_limits()
    L, _ = gpu_frame(pt, sc, 1)
    assert pt.device_errors() == 0
    oL, _ = O.PathTracer(sc).render({"max_depth": 8}, 1)
    compare(L[:, :3], oL, "volume frame after the limits are restored")


def test_media_work_order_keeps_the_frame(krr_lib, cuda):
    """Tracking items taken by estimated optical depth or in queue order:
    the same frame bit for bit."""
    sc = scenes.volume_box(80, 64, max_depth=10, grid=48)
    imgs = []
    for order in (1, 0):
        pt = WavefrontPathTracer({"max_depth": 10})
        pt.set_media_order(order)
        pt.set_scene(sc)
        pt.resize(sc.width, sc.height)
        pt.begin_frame(3, sc.camera)
        imgs.append(pt.render().cpu().numpy())
        assert pt.device_errors() == 0
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
