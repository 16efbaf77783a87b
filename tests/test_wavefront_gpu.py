"""Wavefront path tracer on the GPU against the CPU restatement (per pixel).

Tolerance: per pixel and channel |gpu - oracle| <= 1e-4 * |oracle| + 1e-6.
The shading code rounds every float operation as written on both sides, so
differences come only from CUDA's vs glibc's transcendental functions
(<= 2 ulp); a pixel whose path takes another branch because of such an ulp
is an outlier, and at most 0.2% of pixels may be outliers.  How far the
outliers are off is bounded too: the absolute differences of the whole frame
sum to at most 0.5% of its radiance, the frame's mean radiance agrees within
0.5%, and on frames of 65,536 pixels or more the relMSE of the frame against
the oracle (the reference's metric, per pixel clamped at 100,
src/render/passes/errormeasure/metrics.cu:80-90) stays below 2e-3."""
import numpy as np
import pytest
import torch

from kiraray_gb300 import scenes
from kiraray_gb300.wavefront import WavefrontPathTracer
from oracle import pyoracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu

RTOL, ATOL, MAX_OUTLIERS = 1e-4, 1e-6, 0.002
MAX_FRAME_RELMSE, MAX_MEAN_REL, MAX_L1_REL = 2e-3, 5e-3, 5e-3


def frame_relmse(g, o):
    """relMSE of frame g against o: per channel ((g - o) / o)^2, 0 where o
    is 0, mean over channels, clamped at 100 per pixel, mean over pixels."""
    with np.errstate(divide="ignore", invalid="ignore"):
        e = np.where(o == 0, 0.0, ((g - o) / o) ** 2)
    return float(np.minimum(e.mean(1), 100.0).mean())


def compare(gpu_L, ora_L, what, max_outliers=MAX_OUTLIERS):
    g = gpu_L.astype(np.float64)
    o = ora_L.astype(np.float64)
    bad = np.abs(g - o) > RTOL * np.abs(o) + ATOL
    bad_px = bad.any(axis=1)
    frac = bad_px.mean()
    assert np.isfinite(g).all(), f"{what}: non-finite radiance"
    rel = frame_relmse(g, o)
    mean_rel = abs(g.mean() - o.mean()) / max(abs(o.mean()), 1e-30)
    l1_rel = np.abs(g - o).sum() / max(np.abs(o).sum(), 1e-30)
    with np.errstate(divide="ignore", invalid="ignore"):
        worst = np.nanmax(np.where(bad, np.abs(g - o) / np.abs(o), 0.0)) if bad.any() else 0.0
    print(f"[parity] {what}: outliers {bad_px.sum()}/{bad_px.size}, frame relMSE {rel:.3g}, "
          f"mean rel {mean_rel:.3g}, L1 rel {l1_rel:.3g}, worst outlier rel {worst:.3g}")
    assert frac <= max_outliers, (f"{what}: {bad_px.sum()} of {bad_px.size} pixels differ "
                                  f"(first {np.where(bad_px)[0][:5]}, gpu {g[bad_px][:3]}, "
                                  f"oracle {o[bad_px][:3]})")
    assert l1_rel <= MAX_L1_REL, f"{what}: outliers too far off: L1 difference {l1_rel:.3g} of the frame"
    assert mean_rel <= MAX_MEAN_REL, f"{what}: frame mean differs by {mean_rel:.3g}"
    if g.shape[0] >= 65536:
        assert rel <= MAX_FRAME_RELMSE, f"{what}: outliers too far off: frame relMSE {rel:.3g}"
    return frac


def gpu_frame(pt, sc, frame):
    pt.begin_frame(frame, sc.camera)
    img = pt.render()
    L = pt.radiance()
    torch.cuda.synchronize()
    return L.cpu().numpy(), img.cpu().numpy()


@pytest.mark.parametrize("frame", [1, 2, 7])
def test_cornell_box_per_pixel(krr_lib, cuda, frame):
    sc = scenes.cornell_box(128, 128, max_depth=5)
    pt = WavefrontPathTracer({"max_depth": 5})
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    L, img = gpu_frame(pt, sc, frame)
    oL, opx = O.PathTracer(sc).render({"max_depth": 5}, frame)
    compare(L[:, :3], oL, f"cornell frame {frame}")
    # render() output: pixel / spp, row 0 at the top
    want = opx.reshape(sc.height, sc.width, 3)[::-1]
    got = img[..., :3]
    assert np.mean(np.abs(got - want) > RTOL * np.abs(want) + ATOL) < 3 * MAX_OUTLIERS
    assert np.all(img[..., 3] == 1.0)
    assert pt.device_errors() == 0
    assert (L[:, :3].sum(1) > 0).mean() > 0.4


def test_cornell_box_no_nee_and_clamp(krr_lib, cuda):
    sc = scenes.cornell_box(96, 96, max_depth=4)
    params = {"max_depth": 4, "nee": False, "enable_clamp": True, "clamp_max": 2.0}
    pt = WavefrontPathTracer(params)
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    L, img = gpu_frame(pt, sc, 3)
    oL, _ = O.PathTracer(sc).render(params, 3)
    compare(L[:, :3], oL, "cornell without NEE")
    assert img[..., :3].max() <= 2.0


def test_large_scene_materials_and_environment(krr_lib, cuda):
    sc = scenes.large_scene(width=192, height=108, grid=192, n_spheres=60, sky_size=(256, 128),
                            max_depth=8)
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    L, _ = gpu_frame(pt, sc, 1)
    oL, _ = O.PathTracer(sc).render({"max_depth": 8}, 1)
    compare(L[:, :3], oL, "large scene")
    assert pt.device_errors() == 0


def test_spp_and_seed(krr_lib, cuda):
    sc = scenes.cornell_box(64, 64, max_depth=3)
    pt = WavefrontPathTracer({"max_depth": 3}, spp=3, seed=11)
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    pt.begin_frame(2, sc.camera)
    img = pt.render().cpu().numpy()
    _, opx = O.PathTracer(sc).render({"max_depth": 3}, 2, spp=3, seed=11)
    want = (opx / 3.0).reshape(64, 64, 3)[::-1]
    bad = np.abs(img[..., :3] - want) > RTOL * np.abs(want) + ATOL
    assert bad.any(axis=2).mean() <= MAX_OUTLIERS


def test_independent_samples(krr_lib, cuda):
    """independent_samples=1: L cleared between the samples of a frame; the
    default keeps the reference's running sum, so the two frames differ."""
    sc = scenes.cornell_box(48, 48, max_depth=3)
    imgs = {}
    for ind in (0, 1):
        pt = WavefrontPathTracer({"max_depth": 3, "independent_samples": ind}, spp=4, seed=5)
        pt.set_scene(sc)
        pt.resize(sc.width, sc.height)
        pt.begin_frame(3, sc.camera)
        imgs[ind] = pt.render().cpu().numpy()
        _, opx = O.PathTracer(sc).render({"max_depth": 3, "independent_samples": ind}, 3,
                                         spp=4, seed=5)
        want = (opx / 4.0).reshape(48, 48, 3)[::-1]
        bad = np.abs(imgs[ind][..., :3] - want) > RTOL * np.abs(want) + ATOL
        assert bad.any(axis=2).mean() <= MAX_OUTLIERS
    # running sums weigh the first sample 4x: the mean is ~2.5x the independent one
    ratio = imgs[0][..., :3].mean() / imgs[1][..., :3].mean()
    assert 1.8 < ratio < 3.2


def test_stage_api_and_queue_sizes(krr_lib, cuda):
    sc = scenes.cornell_box(32, 32)
    pt = WavefrontPathTracer({"max_depth": 5})
    pt.set_scene(sc)
    pt.resize(32, 32)
    pt.begin_frame(1, sc.camera)
    pt.reset_queues(-1)
    pt.generate_camera_rays()
    assert pt.queue_size(0) == 32 * 32
    pt.reset_queues(0)
    pt.trace_closest(0)
    n_scatter, n_miss = pt.queue_size(5), pt.queue_size(2)
    assert n_scatter + n_miss <= 32 * 32 and n_scatter > 0
    pt.handle_hit()
    pt.handle_miss()
    pt.generate_scatter_rays(0)
    assert pt.queue_size(1) <= n_scatter
    shadow = pt.queue_items(4)
    assert shadow.shape[1:] == (5, 4) and shadow.shape[0] == pt.queue_size(4)
    if shadow.shape[0]:
        # shadow rays end on the light sample: tMax = 1 (spawnRayTo)
        assert torch.all(shadow[:, 1, 3] == 1.0)
    pt.trace_shadow()
    assert pt.device_errors() == 0


def test_render_equals_stage_loop(krr_lib, cuda):
    """render() traces each bounce's shadow rays together with the next
    bounce's rays; the radiance must equal the stage-by-stage loop of
    integrator.cpp:223-254 bit for bit."""
    sc = scenes.large_scene(width=96, height=64, grid=256, n_spheres=40, sky_size=(64, 32))
    depth_max = 6
    pt = WavefrontPathTracer({"max_depth": depth_max}, seed=4)
    pt.set_scene(sc)
    pt.resize(96, 64)
    pt.begin_frame(2, sc.camera)
    pt.render()
    fused = pt.radiance().cpu().numpy()
    pt.begin_frame(2, sc.camera)
    pt.reset_queues(-1)
    pt.generate_camera_rays()
    for d in range(depth_max + 1):
        pt.reset_queues(d)
        pt.trace_closest(d)
        pt.handle_hit()
        pt.handle_miss()
        if d == depth_max:
            break
        pt.generate_scatter_rays(d)
        pt.trace_shadow()
    staged = pt.radiance().cpu().numpy()
    assert np.array_equal(fused.view(np.uint32), staged.view(np.uint32))
    assert pt.device_errors() == 0


def test_resize_and_rescene(krr_lib, cuda):
    pt = WavefrontPathTracer({"max_depth": 2})
    sc = scenes.cornell_box(40, 30)
    pt.set_scene(sc)
    for w, h in ((40, 30), (17, 23)):
        pt.resize(w, h)
        pt.begin_frame(1, sc.camera)
        img = pt.render()
        assert img.shape == (h, w, 4) and torch.isfinite(img).all()
    pt.set_scene(scenes.cornell_box(17, 23))
    pt.begin_frame(2, sc.camera)
    assert torch.isfinite(pt.render()).all()


@pytest.mark.parametrize("reorder", [1, 0])
@pytest.mark.parametrize("params,spp", [({"max_depth": 5}, 1), ({"max_depth": 3, "nee": False}, 1),
                                        ({"max_depth": 4, "enable_clamp": True, "clamp_max": 1.5}, 2),
                                        ({"max_depth": 4, "independent_samples": 1}, 3)])
def test_megakernel_equals_wavefront_cornell(krr_lib, cuda, params, spp, reorder):
    """The megakernel, with and without regrouping paths by hit class after
    each closest hit, equals the wavefront bit for bit."""
    sc = scenes.cornell_box(64, 48, max_depth=params["max_depth"])
    pt = WavefrontPathTracer(params, spp=spp, seed=9)
    pt.set_megakernel_reorder(reorder)
    pt.set_scene(sc)
    pt.resize(64, 48)
    pt.begin_frame(4, sc.camera)
    a = pt.render().cpu().numpy()
    La = pt.radiance().cpu().numpy()
    pt.begin_frame(4, sc.camera)
    b = pt.render_megakernel().cpu().numpy()
    Lb = pt.radiance().cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(La.view(np.uint32), Lb.view(np.uint32))
    assert pt.device_errors() == 0


@pytest.mark.parametrize("reorder", [1, 0])
def test_megakernel_equals_wavefront_large_scene_views(krr_lib, cuda, reorder):
    """Conductors, dielectrics, the environment and two batched views (view
    sizes not multiples of the 128-path blocks)."""
    sc = scenes.large_scene(width=96, height=64, grid=256, n_spheres=40, sky_size=(64, 32))
    views = [(sc.camera, 96, 64, 3), (sc.camera, 40, 30, 1 << 24)]
    pt = WavefrontPathTracer({"max_depth": 8})
    pt.set_megakernel_reorder(reorder)
    pt.set_scene(sc)
    pt.resize_views(views)
    pt.begin_frame_views(2)
    a = pt.render_flat().cpu().numpy()
    out = torch.empty((pt.n_pixels, 4), device="cuda")
    pt.begin_frame_views(2)
    pt.render_megakernel(out)
    b = out.cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_megakernel_rejects_media(krr_lib, cuda):
    from kiraray_gb300._lib import KrrError
    sc = scenes.volume_box(16, 16)
    pt = WavefrontPathTracer({"max_depth": 3})
    pt.set_scene(sc)
    pt.resize(16, 16)
    pt.begin_frame(1, sc.camera)
    with pytest.raises(KrrError):
        pt.render_megakernel()


def test_update_instances_equals_fresh_scene(krr_lib, cuda):
    """Animated instances: moving instances (boxes refitted over the existing
    tree) gives the frame a pass built from the moved scene renders, bit for
    bit; so do a full rebuild afterwards and moving them back."""
    import copy
    sc = scenes.large_scene(width=64, height=48, grid=128, n_spheres=12, sky_size=(64, 32))
    moved = copy.deepcopy(sc)
    idx = [len(sc.instances) - 1, 3]   # an emissive quad and a sphere
    xfs = []
    for k in idx:
        mesh, xf = moved.instances[k]
        xf = np.array(xf, np.float32)
        xf[:, 3] += np.array([0.7, 0.2, -0.4], np.float32)
        moved.instances[k] = (mesh, xf)
        xfs.append(xf)
    pt = WavefrontPathTracer({"max_depth": 6})
    pt.set_scene(sc)
    pt.resize(64, 48)
    pt.update_instances(idx, np.stack(xfs))
    pt.begin_frame(3, sc.camera)
    a = pt.render().cpu().numpy()
    fresh = WavefrontPathTracer({"max_depth": 6})
    fresh.set_scene(moved)
    fresh.resize(64, 48)
    fresh.begin_frame(3, moved.camera)
    b = fresh.render().cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    pt.rebuild_bvh()
    pt.begin_frame(3, sc.camera)
    assert np.array_equal(pt.render().cpu().numpy().view(np.uint32), b.view(np.uint32))
    pt.update_instances(idx, np.stack([np.array(sc.instances[k][1], np.float32) for k in idx]))
    pt.begin_frame(3, sc.camera)
    back = pt.render().cpu().numpy()
    orig = WavefrontPathTracer({"max_depth": 6})
    orig.set_scene(sc)
    orig.resize(64, 48)
    orig.begin_frame(3, sc.camera)
    assert np.array_equal(back.view(np.uint32), orig.render().cpu().numpy().view(np.uint32))
    assert pt.device_errors() == 0


def test_scene_without_emitters_and_tiny_frames(krr_lib, cuda):
    """No area or infinite light: NEE has nothing to sample and the frame is
    black; frames of 1x1 and 3x1 pixels; both match the oracle."""
    from kiraray_gb300.scenes import Material
    dark = scenes.cornell_box(8, 8, max_depth=4)
    for m in dark.meshes:
        m.emission = (0.0, 0.0, 0.0)
    dark.infinite_lights = []
    pt = WavefrontPathTracer({"max_depth": 4})
    pt.set_scene(dark)
    for w, h in ((8, 8), (1, 1), (3, 1)):
        pt.resize(w, h)
        pt.begin_frame(2, dark.camera)
        img = pt.render().cpu().numpy()
        assert img.shape == (h, w, 4) and np.all(img[..., :3] == 0.0)
        b = pt.render_megakernel().cpu().numpy()
        assert np.all(b[..., :3] == 0.0)
    assert pt.device_errors() == 0
    lit = scenes.cornell_box(3, 1, max_depth=4)
    pt.set_scene(lit)
    pt.resize(3, 1)
    L, _ = gpu_frame(pt, lit, 5)
    oL, _ = O.PathTracer(lit).render({"max_depth": 4}, 5)
    compare(L[:, :3], oL, "3x1 frame")


def test_empty_geometry(krr_lib, cuda):
    """No triangles: every ray misses; the frame is the environment."""
    from kiraray_gb300.accel import Accel
    from kiraray_gb300.scenes import InfiniteLight, Material, Scene
    acc = Accel(np.zeros((0, 9), np.float32))
    one = np.array([[0, 0, 0, 0, 0, 0, 1, np.inf]], np.float32)
    rays = torch.from_numpy(np.tile(one, (100, 1))).cuda()
    hits = acc.trace_closest(rays).cpu().numpy()
    assert np.all(hits[:, 3].view(np.uint32) == 0xFFFFFFFF) and np.all(np.isinf(hits[:, 0]))
    assert not acc.trace_any(rays).cpu().numpy().any()
    cam = scenes.cornell_box(16, 12).camera
    sc = Scene([], [], [Material()], cam, 16, 12,
               infinite_lights=[InfiniteLight(tint=(0.2, 0.3, 0.5), scale=2.0)], max_depth=3)
    pt = WavefrontPathTracer({"max_depth": 3})
    pt.set_scene(sc)
    pt.resize(16, 12)
    pt.begin_frame(1, cam)
    img = pt.render().cpu().numpy()
    assert np.allclose(img[..., :3], np.array([0.4, 0.6, 1.0], np.float32), rtol=1e-6)
    assert pt.device_errors() == 0


def test_two_level_structure_in_the_pass(krr_lib, cuda):
    """The pass on the two-level structure (each geometry once, an instance
    tree over them): frames within the per-pixel tolerance of the oracle
    (object-space hits differ from world-space ones by rounding), and after
    an instance update (only the instance tree is rebuilt) equal bit for bit
    to a two-level pass built from the moved scene."""
    import copy
    sc = scenes.large_scene(width=160, height=90, grid=128, n_spheres=40, sky_size=(128, 64),
                            max_depth=6)
    pt = WavefrontPathTracer({"max_depth": 6})
    pt.set_accel_levels(2)
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    L, _ = gpu_frame(pt, sc, 2)
    assert pt.device_errors() == 0
    oL, _ = O.PathTracer(sc).render({"max_depth": 6}, 2)
    compare(L[:, :3], oL, "two-level large scene", max_outliers=0.01)
    moved = copy.deepcopy(sc)
    xfs = []
    for k in (3, 10, 17):
        mesh, xf = moved.instances[k]
        xf = np.array(xf, np.float32)
        xf[:, 3] += np.array([0.5, 0.3, -0.4], np.float32)
        moved.instances[k] = (mesh, xf)
        xfs.append(xf)
    pt.update_instances([3, 10, 17], np.stack(xfs))
    got, _ = gpu_frame(pt, moved, 3)
    ref = WavefrontPathTracer({"max_depth": 6})
    ref.set_accel_levels(2)
    ref.set_scene(moved)
    ref.resize(sc.width, sc.height)
    want, _ = gpu_frame(ref, moved, 3)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # the volume box (null-material interface, medium tracking) on two levels
    vb = scenes.volume_box(64, 64, max_depth=8, grid=32)
    pv = WavefrontPathTracer({"max_depth": 8})
    pv.set_accel_levels(2)
    pv.set_scene(vb)
    pv.resize(64, 64)
    L, _ = gpu_frame(pv, vb, 1)
    assert pv.device_errors() == 0
    oL, _ = O.PathTracer(vb).render({"max_depth": 8}, 1)
    compare(L[:, :3], oL, "two-level volume box", max_outliers=0.01)


@pytest.mark.parametrize("nee", [1, 0])
def test_closed_lambertian_sphere_radiance(krr_lib, cuda, nee):
    """Known answer through the CUDA pass: inside a closed sphere that emits
    Le and reflects with Lambertian albedo a, every pixel converges to
    Le (1 - a^(D+1)) / (1 - a)."""
    sc, want = H.furnace_sphere()
    pt = WavefrontPathTracer({"max_depth": sc.max_depth, "nee": nee})
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    acc = torch.zeros(3, dtype=torch.float64, device="cuda")
    frames = 64
    for f in range(1, frames + 1):
        pt.begin_frame(f, sc.camera)
        acc += pt.render()[..., :3].reshape(-1, 3).double().mean(0)
    got = (acc / frames).cpu().numpy()
    np.testing.assert_allclose(got, want, rtol=0.02)
    assert pt.device_errors() == 0


def test_stage_timers(krr_lib, cuda):
    """Per-stage device timers (the reference's PROFILE events): off by
    default, named after the reference's stages, counted per launch, reset by
    each read, skipped while a frame is captured into a graph, and without
    effect on the frame."""
    sc = scenes.large_scene(width=64, height=48, grid=128, n_spheres=20, sky_size=(64, 32))
    pt = WavefrontPathTracer({"max_depth": 4})
    pt.set_scene(sc)
    pt.resize(64, 48)
    pt.begin_frame(1, sc.camera)
    want = pt.render().cpu().numpy()
    assert pt.profile() == {}
    pt.set_profiling(True)
    for f in (1, 2):
        pt.begin_frame(f, sc.camera)
        got = pt.render()
        if f == 1:
            assert np.array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32))
    prof = pt.profile()
    assert prof["Begin frame"][0] == 2 and prof["Generate camera rays"][0] == 2
    assert prof["Trace intersect rays"][0] == 2          # camera rays; later bounces go with the shadows
    assert prof["Trace shadow and next rays"][0] >= 2
    assert prof["Route closest hits"][0] >= 4 and prof["Generate scatter rays"][0] >= 4
    assert prof["Accumulate and resolve"][0] == 4
    assert all(ms >= 0 for _, ms in prof.values()) and sum(ms for _, ms in prof.values()) > 0
    assert pt.profile() == {}
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        out = torch.empty((48, 64, 4), device="cuda")
        pt.capture_frame(out)
        pt.launch_frame(3)
        s.synchronize()
        assert pt.profile() == {}
    pt.set_profiling(False)
    pt.begin_frame(4, sc.camera)
    pt.render()
    assert pt.profile() == {}
    # a pass with media times its tracking stages
    vol = scenes.volume_box(32, 32, max_depth=6, grid=32)
    pv = WavefrontPathTracer({"max_depth": 6})
    pv.set_scene(vol)
    pv.resize(32, 32)
    pv.set_profiling(True)
    pv.begin_frame(1, vol.camera)
    pv.render()
    pm = pv.profile()
    assert pm["Sample medium interaction"][0] >= 1 and pm["Trace shadow rays"][0] >= 1
    assert pt.device_errors() == 0 and pv.device_errors() == 0

