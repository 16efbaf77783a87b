"""Batched views in one wavefront and CUDA-graph frame replay.

Every stage computes each pixel independently, so a view rendered inside a
batch must equal the same view rendered alone with the same seed, bit for
bit, and a replayed graph must equal an ordinary frame."""

import numpy as np
import pytest
import torch

from kiraray_gb300 import scenes
from kiraray_gb300.nrc import NeuralRadianceCache
from kiraray_gb300.wavefront import WavefrontPathTracer

pytestmark = pytest.mark.gpu


def _views():
    sc = scenes.cornell_box(8, 8)
    out = []
    for i, (w, h) in enumerate(((48, 32), (17, 29), (64, 64))):
        cam = scenes._camera((0.5 + 0.05 * i, 0.5, -1.4), (0.5, 0.45, 0.0), 40.0 - 5 * i, w, h)
        out.append((cam, w, h, 100 + i))
    return sc, out


def test_graph_replay_after_instance_update(krr_lib, cuda):
    """An instance update refits the BVH in place, so a frame captured before
    it replays the moved scene: equal to an ordinary frame of a pass built
    from the moved scene."""
    import copy
    sc, views = _views()
    moved = copy.deepcopy(sc)
    mesh, xf = moved.instances[6]
    xf = np.array(xf, np.float32)
    xf[:, 3] += np.array([0.08, 0.0, -0.05], np.float32)
    moved.instances[6] = (mesh, xf)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        pt = WavefrontPathTracer({"max_depth": 5})
        pt.set_scene(sc)
        pt.resize_views(views)
        out = torch.empty((pt.n_pixels, 4), device="cuda")
        pt.begin_frame_views(1)
        pt.render_flat(out)
        pt.capture_frame(out)
        pt.update_instances([6], xf[None])
        pt.launch_frame(2)
        s.synchronize()
        got = out.cpu().numpy().copy()
        ref = WavefrontPathTracer({"max_depth": 5})
        ref.set_scene(moved)
        ref.resize_views(views)
        ref.begin_frame_views(2)
        want = ref.render_flat().cpu().numpy()
        s.synchronize()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert pt.device_errors() == 0


def test_batched_views_equal_single_views(krr_lib, cuda):
    sc, views = _views()
    pt = WavefrontPathTracer({"max_depth": 5})
    pt.set_scene(sc)
    pt.resize_views(views)
    pt.begin_frame_views(3)
    batch = pt.render_flat().cpu().numpy()
    off = 0
    for cam, w, h, seed in views:
        single = WavefrontPathTracer({"max_depth": 5}, seed=seed)
        single.set_scene(sc)
        single.resize(w, h)
        single.begin_frame(3, cam)
        img = single.render().cpu().numpy().reshape(-1, 4)
        assert np.array_equal(batch[off:off + w * h].view(np.uint32), img.view(np.uint32))
        off += w * h
    assert pt.device_errors() == 0


def test_graph_replay_equals_ordinary_frames(krr_lib, cuda):
    sc, views = _views()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        pt = WavefrontPathTracer({"max_depth": 5})
        pt.set_scene(sc)
        pt.resize_views(views)
        out = torch.empty((pt.n_pixels, 4), device="cuda")
        pt.begin_frame_views(1)
        pt.render_flat(out)
        pt.capture_frame(out)
        got = []
        for f in (2, 3, 4):
            pt.launch_frame(f)
            s.synchronize()
            got.append(out.cpu().numpy().copy())
        ref = WavefrontPathTracer({"max_depth": 5})
        ref.set_scene(sc)
        ref.resize_views(views)
        for k, f in enumerate((2, 3, 4)):
            ref.begin_frame_views(f)
            want = ref.render_flat().cpu().numpy()
            assert np.array_equal(got[k].view(np.uint32), want.view(np.uint32)), f
    assert not np.array_equal(got[0], got[1])


def test_graph_replay_with_cache_training(krr_lib, cuda):
    sc, views = _views()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        pt = WavefrontPathTracer({"max_depth": 5})
        pt.set_scene(sc)
        pt.resize_views(views)
        cache = NeuralRadianceCache((0, 0, 0), (1, 1, 1), batch_size=4096)
        pt.set_nrc(cache, train=True)
        out = torch.empty((pt.n_pixels, 4), device="cuda")
        pt.begin_frame_views(1)
        pt.render_flat(out)
        pt.capture_frame(out)
        for f in range(2, 12):
            pt.launch_frame(f)
        s.synchronize()
    assert cache.info().step == 11
    assert torch.isfinite(out).all()
    assert pt.device_errors() == 0


def test_single_view_graph_replay_advances_samples(krr_lib, cuda):
    """resize() + begin_frame(camera) + capture; replays without new cameras
    keep the camera and seed and move to the frame's sample index."""
    sc = scenes.cornell_box(24, 16, max_depth=4)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        pt = WavefrontPathTracer({"max_depth": 4}, seed=7)
        pt.set_scene(sc)
        pt.resize(24, 16)
        out = torch.empty((16, 24, 4), device="cuda")
        pt.begin_frame(1, sc.camera)
        pt.render(out)
        pt.capture_frame(out)
        got = {}
        for f in (5, 6):
            pt.launch_frame(f)
            s.synchronize()
            got[f] = out.cpu().numpy().copy()
        ref = WavefrontPathTracer({"max_depth": 4}, seed=7)
        ref.set_scene(sc)
        ref.resize(24, 16)
        for f in (5, 6):
            ref.begin_frame(f, sc.camera)
            want = ref.render().cpu().numpy()
            assert np.array_equal(got[f].view(np.uint32), want.view(np.uint32)), f
    assert not np.array_equal(got[5], got[6])


def test_frame_group_equals_passes_alone(krr_lib, cuda):
    """Two scenes (surfaces with views, volume box with views) captured as one
    graph with a branch per pass; each output equals its pass rendered alone."""
    from kiraray_gb300.wavefront import FrameGroup
    sc_a, views_a = _views()
    sc_b = scenes.volume_box(8, 8, grid=32)
    views_b = [(sc_b.camera, 24, 24, 7), (sc_b.camera, 16, 12, 1 << 24)]
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        pa = WavefrontPathTracer({"max_depth": 5})
        pa.set_scene(sc_a)
        pa.resize_views(views_a)
        pb = WavefrontPathTracer({"max_depth": 6})
        pb.set_scene(sc_b)
        pb.resize_views(views_b)
        oa = torch.empty((pa.n_pixels, 4), device="cuda")
        ob = torch.empty((pb.n_pixels, 4), device="cuda")
        for p, o in ((pa, oa), (pb, ob)):
            p.begin_frame_views(1)
            p.render_flat(o)
        grp = FrameGroup([pa, pb], [oa, ob])
        grp.capture()
        got = {}
        for f in (3, 4):
            grp.launch(f)
            s.synchronize()
            got[f] = (oa.cpu().numpy().copy(), ob.cpu().numpy().copy())
        for f in (3, 4):
            for k, (p, sc, views) in enumerate(((pa, sc_a, views_a), (pb, sc_b, views_b))):
                ref = WavefrontPathTracer({"max_depth": 5 if k == 0 else 6})
                ref.set_scene(sc)
                ref.resize_views(views)
                ref.begin_frame_views(f)
                want = ref.render_flat().cpu().numpy()
                assert np.array_equal(got[f][k].view(np.uint32), want.view(np.uint32)), (f, k)
        grp.close()
    assert pa.device_errors() == 0 and pb.device_errors() == 0


def _two_scene_views():
    big = scenes.large_scene(width=8, height=8, grid=128, n_spheres=30, sky_size=(64, 32))
    vol = scenes.volume_box(8, 8, max_depth=8, grid=32)
    views = []
    for i, (w, h) in enumerate(((40, 24), (33, 21), (24, 40), (16, 16))):
        if i % 2 == 0:
            cam = scenes._camera((3.0 * i, 22.0, -62.0), (0.0, 2.0, 0.0), 45.0, w, h)
        else:
            cam = scenes._camera((0.5 + 0.1 * i, 0.5, -1.4), (0.5, 0.5, 0.0), 40.0, w, h)
        views.append((cam, w, h, 200 + i, i % 2))
    return [big, vol], views


def _alone(sc, view, frame, max_depth):
    cam, w, h, seed = view[:4]
    pt = WavefrontPathTracer({"max_depth": max_depth})
    pt.set_scene(sc)
    pt.resize_views([(cam, w, h, seed)])
    pt.begin_frame_views(frame)
    out = pt.render_flat().cpu().numpy()
    assert pt.device_errors() == 0
    return out


def test_scenes_in_one_wavefront_equal_each_scene_alone(krr_lib, cuda):
    """Views of two scenes (the large scene without media at max depth 8, the
    volume box with a medium at max depth 12) in one pass: one launch per
    stage per bounce serves both, and every view equals its scene's pass
    rendering that view alone."""
    (big, vol), views = _two_scene_views()
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_scenes([big, vol])
    pt.set_scene_max_depth(1, 12)
    pt.resize_views(views)
    pt.begin_frame_views(2)
    batch = pt.render_flat().cpu().numpy()
    assert pt.device_errors() == 0
    off = 0
    for v in views:
        w, h = v[1], v[2]
        want = _alone((big, vol)[v[4]], v, 2, (8, 12)[v[4]])
        assert np.array_equal(batch[off:off + w * h].view(np.uint32), want.view(np.uint32)), v[4]
        off += w * h
    # a view naming a scene the pass does not hold is rejected
    with pytest.raises(Exception):
        pt.resize_views([(views[0][0], 8, 8, 1, 2)])


def test_launch_shapes_and_waves_keep_the_frame(krr_lib, cuda):
    """Threads per block, blocks per SM and waves of pixels (queue capacity
    below the pixel count) change nothing in the frame."""
    (big, vol), views = _two_scene_views()
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_scenes([big, vol])
    pt.resize_views(views)
    pt.begin_frame_views(3)
    want = pt.render_flat().cpu().numpy()
    n = pt.n_pixels
    for block, bps, wave in ((128, 4, 0), (64, 16, n // 3 + 5), (256, 2, 1000)):
        pt.set_launch(block, bps, wave)
        assert pt.launch()["queue_capacity"] == (min(wave, n) if wave else n)
        pt.begin_frame_views(3)
        got = pt.render_flat().cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (block, bps, wave)
    assert pt.device_errors() == 0
    with pytest.raises(Exception):   # the stage entry points need every pixel in the queues
        pt.generate_camera_rays()


def test_camera_order_keeps_the_frame(krr_lib, cuda):
    """Camera rays queued in 8x8 pixel tiles (the default) or row-major give
    the same frame bit for bit, with views whose sizes are not multiples of
    eight and with waves that end inside a view."""
    (big, vol), views = _two_scene_views()
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_scenes([big, vol])
    pt.resize_views(views)
    pt.set_camera_order(False)
    pt.begin_frame_views(5)
    want = pt.render_flat().cpu().numpy()
    n = pt.n_pixels
    pt.set_camera_order(True)
    for wave in (0, n // 3 + 5, 999):
        pt.set_launch(256, 8, wave)
        pt.begin_frame_views(5)
        got = pt.render_flat().cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), wave
    assert pt.device_errors() == 0
    from kiraray_gb300._lib import KrrError, check
    with pytest.raises(KrrError):
        check(pt.lib.krr_wf_set_camera_order(pt._h, 2), "krr_wf_set_camera_order")


def test_autotuner_keeps_the_frame(krr_lib, cuda):
    (big, vol), views = _two_scene_views()
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_scenes([big, vol])
    pt.resize_views(views)
    pt.begin_frame_views(4)
    want = pt.render_flat().cpu().numpy()
    out = torch.empty((pt.n_pixels, 4), device="cuda")
    t = pt.autotune(out, frames=2)
    assert t["candidates"] == 6 and t["frame_ms"] > 0
    assert t["frame_ms"] <= t["default_frame_ms"]
    assert pt.launch()["block"] == t["block"]
    pt.begin_frame_views(4)
    got = pt.render_flat().cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_cache_across_scenes_in_one_wavefront(krr_lib, cuda):
    """One cache for both scenes: their positions are offset into disjoint
    regions of the cache's box; frames stay finite and the cache trains."""
    (big, vol), views = _two_scene_views()
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_scenes([big, vol])
    pt.resize_views(views)
    lo, hi = pt.cache_box()
    assert hi[0] - lo[0] > 100.0   # the volume box sits beside the large scene
    cache = NeuralRadianceCache(lo, hi, batch_size=2048)
    pt.set_nrc(cache, train=True)
    for f in range(1, 6):
        pt.begin_frame_views(f)
        img = pt.render_flat()
    assert torch.isfinite(img).all()
    assert cache.info().step == 5
    assert pt.device_errors() == 0
