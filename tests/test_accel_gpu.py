"""GPU closest-hit / any-hit parity against the CPU oracle (bit-exact).

The hit record (t, b1, b2, triangle id) of the CUDA traversal must equal the
oracle's bit for bit: both run the same watertight test with the same
rounding, and ties in t go to the smaller triangle id on both sides."""
import numpy as np
import pytest
import torch

from kiraray_gb300 import scenes
from kiraray_gb300.accel import Accel
from oracle import pyoracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _gpu_closest(acc, rays):
    out = acc.trace_closest(torch.from_numpy(rays).cuda())
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _assert_bits_equal(a, b, what):
    ua, ub = a.view(np.uint32), b.view(np.uint32)
    bad = np.where(~np.all(ua == ub, axis=1))[0]
    assert bad.size == 0, f"{what}: {bad.size} of {a.shape[0]} hits differ, first {bad[:5]}: " \
                          f"gpu {a[bad[:3]]} oracle {b[bad[:3]]}"


def test_cornell_box_camera_rays(krr_lib, cuda):
    sc = scenes.cornell_box()
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc)
    acc = Accel(tris)
    got = _gpu_closest(acc, rays)
    want = O.Bvh(tris).closest(rays)
    _assert_bits_equal(got, want, "cornell camera rays")
    assert (got[:, 3].view(np.uint32) != 0xFFFFFFFF).mean() > 0.9


@pytest.mark.parametrize("n_tris,seed", [(1, 0), (2, 1), (3, 2), (4, 3), (5, 9), (100, 4),
                                         (5000, 5), (60000, 6)])
def test_random_soup_vs_brute_force(krr_lib, cuda, n_tris, seed):
    tris = H.random_soup(n_tris, seed, size=0.2 if n_tris > 100 else 1.0)
    rays = H.random_rays(3000, seed + 50)
    acc = Accel(tris)
    got = _gpu_closest(acc, rays)
    want = O.closest_brute(tris, rays) if n_tris <= 5000 else O.Bvh(tris).closest(rays)
    _assert_bits_equal(got, want, f"soup {n_tris}")


def test_shared_vertices_and_edges_do_not_leak(krr_lib, cuda):
    tris = H.grid_mesh(16)
    rays = H.vertex_edge_rays(16, 7)
    acc = Accel(tris)
    got = _gpu_closest(acc, rays)
    assert np.all(got[:, 3].view(np.uint32) != 0xFFFFFFFF)
    _assert_bits_equal(got, O.closest_brute(tris, rays), "grid vertex/edge rays")


def test_closed_mesh_from_inside(krr_lib, cuda):
    m = scenes.icosphere(4)
    tris = m.positions[m.indices].reshape(-1, 9).astype(np.float32)
    rays = H.random_rays(50000, 11, box=0.0)
    got = _gpu_closest(Accel(tris), rays)
    assert np.all(got[:, 3].view(np.uint32) != 0xFFFFFFFF)


def test_axis_aligned_and_degenerate_directions(krr_lib, cuda):
    sc = scenes.cornell_box()
    tris = sc.world_triangles()
    rng = np.random.default_rng(3)
    dirs = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [0, 0, 0], [1e-30, 0, 1], [-0.0, 1, 0]], np.float32)
    o = rng.random((400, 3)).astype(np.float32) * 0.9 + 0.05
    rays = np.zeros((400 * len(dirs), 8), np.float32)
    rays[:, :3] = np.repeat(o, len(dirs), 0)
    rays[:, 4:7] = np.tile(dirs, (400, 1))
    rays[:, 7] = np.inf
    got = _gpu_closest(Accel(tris), rays)
    _assert_bits_equal(got, O.closest_brute(tris, rays), "axis-aligned rays")


def test_tmin_tmax_and_ties(krr_lib, cuda):
    t = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    tris = np.concatenate([t, t, t, t + np.array([0, 0, -1] * 3, np.float32)])
    rays = np.array([[0.2, 0.2, 1, 0, 0, 0, -1, np.inf],
                     [0.2, 0.2, 1, 1.5, 0, 0, -1, np.inf],
                     [0.2, 0.2, 1, 0, 0, 0, -1, 0.5],
                     [0.2, 0.2, 1, 0, 0, 0, -1, 1.0]], np.float32)
    got = _gpu_closest(Accel(tris), rays)
    assert list(got[:, 3].view(np.uint32)) == [0, 3, 0xFFFFFFFF, 0]
    _assert_bits_equal(got, O.closest_brute(tris, rays), "windows")


def test_any_hit_and_mask(krr_lib, cuda):
    sc = scenes.cornell_box()
    tris = sc.world_triangles()
    rng = np.random.default_rng(8)
    n = 20000
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = rng.random((n, 3)) * 0.9 + 0.05
    rays[:, 4:7] = (rng.random((n, 3)) * 0.9 + 0.05) - rays[:, :3]   # segments, tmax = 1
    rays[:, 7] = 1.0
    acc = Accel(tris)
    occ = acc.trace_any(torch.from_numpy(rays).cuda()).cpu().numpy()
    ob = O.Bvh(tris)
    assert np.array_equal(occ, ob.any(rays))
    mask = np.ones(tris.shape[0], np.uint8)
    mask[10:22] = 0   # the short box does not block
    acc.set_mask(mask)
    ob.set_mask(mask)
    occ2 = acc.trace_any(torch.from_numpy(rays).cuda()).cpu().numpy()
    assert np.array_equal(occ2, ob.any(rays))
    assert occ2.sum() < occ.sum()


def test_empty_ray_batch(krr_lib, cuda):
    acc = Accel(H.random_soup(10, 1))
    out = acc.trace_closest(torch.empty((0, 8), device="cuda"))
    assert out.shape == (0, 4)


def test_host_buffer_entry_point(krr_lib, cuda):
    sc = scenes.cornell_box(64, 64)
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc)
    acc = Accel(tris)
    out = np.zeros((rays.shape[0], 4), np.float32)
    acc.trace_closest_host(rays, out)
    _assert_bits_equal(out, O.Bvh(tris).closest(rays), "host entry point")


def test_large_scene_reduced(krr_lib, cuda):
    sc = scenes.large_scene(width=320, height=180, grid=512, n_spheres=100, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc)
    acc = Accel(tris)
    ob = O.Bvh(tris)
    got = _gpu_closest(acc, rays)
    want = ob.closest(rays)
    _assert_bits_equal(got, want, "large scene camera rays")
    b = H.bounce_rays(tris, rays, want, 5)
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), "large scene bounce rays")
    st = acc.stats()
    assert st["n_triangles"] == tris.shape[0] and st["max_depth"] <= 48


@pytest.mark.slow
def test_full_size_scene_sampled(krr_lib, cuda):
    """10.9M triangles: GPU hits on a 1-in-64 sample of the 1920x1080 camera
    rays and of their first bounce equal the oracle's."""
    sc = scenes.large_scene(sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc)[::64].copy()
    acc = Accel(tris)
    ob = O.Bvh(tris)
    want = ob.closest(rays)
    _assert_bits_equal(_gpu_closest(acc, rays), want, "10M camera rays")
    b = H.bounce_rays(tris, rays, want, 6)
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), "10M bounce rays")


@pytest.mark.parametrize("refill,postpone", [(12, 0), (28, 0), (20, 20), (24, 50)])
def test_tuning_settings_keep_hits_identical(krr_lib, cuda, refill, postpone):
    sc = scenes.large_scene(width=160, height=90, grid=384, n_spheres=80, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=3)
    acc = Accel(tris)
    acc.set_tuning(refill, postpone)
    ob = O.Bvh(tris)
    want = ob.closest(rays)
    _assert_bits_equal(_gpu_closest(acc, rays), want, f"tuning {refill}/{postpone}")
    b = H.bounce_rays(tris, rays, want, 8)
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), f"tuning {refill}/{postpone} bounce")
    occ = acc.trace_any(torch.from_numpy(b).cuda()).cpu().numpy()
    assert np.array_equal(occ, ob.any(b))


def test_autotune_picks_a_setting(krr_lib, cuda):
    sc = scenes.large_scene(width=160, height=90, grid=256, n_spheres=20, sky_size=(64, 32))
    acc = Accel(sc.world_triangles())
    res = acc.autotune(torch.from_numpy(H.pinhole_rays(sc)).cuda(), repeats=1)
    assert 1 <= res["refill_below"] <= 32 and 0 <= res["postpone_pct"] <= 100 and res["ms"] > 0


@pytest.fixture
def float_nodes():
    from kiraray_gb300.accel import set_node_format
    set_node_format(1)
    yield
    set_node_format(0)


@pytest.mark.parametrize("n_tris,seed", [(1, 0), (3, 2), (5, 9), (100, 4), (5000, 5), (60000, 6)])
def test_float_nodes_soup_vs_brute_force(krr_lib, cuda, float_nodes, n_tris, seed):
    tris = H.random_soup(n_tris, seed, size=0.2 if n_tris > 100 else 1.0)
    rays = H.random_rays(3000, seed + 50)
    acc = Accel(tris)
    assert acc.stats()["node_format"] == 1
    want = O.closest_brute(tris, rays) if n_tris <= 5000 else O.Bvh(tris).closest(rays)
    _assert_bits_equal(_gpu_closest(acc, rays), want, f"float nodes soup {n_tris}")


def test_float_nodes_large_scene_and_edges(krr_lib, cuda, float_nodes):
    sc = scenes.large_scene(width=160, height=90, grid=384, n_spheres=80, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=5)
    acc = Accel(tris)
    acc.set_tuning(20, 20)
    ob = O.Bvh(tris)
    want = ob.closest(rays)
    _assert_bits_equal(_gpu_closest(acc, rays), want, "float nodes camera rays")
    b = H.bounce_rays(tris, rays, want, 9)
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), "float nodes bounce rays")
    occ = acc.trace_any(torch.from_numpy(b).cuda()).cpu().numpy()
    assert np.array_equal(occ, ob.any(b))
    g = H.grid_mesh(16)
    r = H.vertex_edge_rays(16, 7)
    _assert_bits_equal(_gpu_closest(Accel(g), r), O.closest_brute(g, r), "float nodes grid edges")


def test_float_nodes_in_wavefront_frame(krr_lib, cuda, float_nodes):
    from kiraray_gb300.wavefront import WavefrontPathTracer
    sc = scenes.cornell_box(32, 32, max_depth=4)
    pt = WavefrontPathTracer({"max_depth": 4})
    pt.set_scene(sc)
    pt.resize(32, 32)
    pt.begin_frame(1, sc.camera)
    pt.render()
    L = pt.radiance().cpu().numpy()[:, :3]
    oL, _ = O.PathTracer(sc).render({"max_depth": 4}, 1)
    bad = (np.abs(L - oL) > 1e-4 * np.abs(oL) + 1e-6).any(1).mean()
    assert bad <= 0.01 and not pt.device_errors()


def test_host_entry_point_pinned_and_pageable(krr_lib, cuda):
    """1.3M host rays from page-locked buffers (traced in place on a coherent
    link, else in chunks) and from pageable arrays (more than four chunks over
    the two streams): the hits equal the device-buffer entry point's."""
    sc = scenes.large_scene(width=160, height=90, grid=256, n_spheres=30, sky_size=(64, 32))
    tris = sc.world_triangles()
    acc = Accel(tris)
    rays = H.random_rays(1_300_000, 77, box=60.0)
    want = _gpu_closest(acc, rays)
    got = torch.empty((rays.shape[0], 4), dtype=torch.float32).pin_memory()
    acc.trace_closest_host(torch.from_numpy(rays).pin_memory(), got)
    _assert_bits_equal(got.numpy(), want, "host entry point, page-locked")
    out = np.zeros((rays.shape[0], 4), np.float32)
    acc.trace_closest_host(np.ascontiguousarray(rays), out)
    _assert_bits_equal(out, want, "host entry point, pageable")
    # mixed: page-locked rays, pageable hits
    out2 = np.zeros((rays.shape[0], 4), np.float32)
    acc.trace_closest_host(torch.from_numpy(rays).pin_memory(), out2)
    _assert_bits_equal(out2, want, "host entry point, mixed")


@pytest.mark.parametrize("node_format", [0, 1])
def test_refit_keeps_hits_exact(krr_lib, cuda, node_format):
    """Boxes refitted over the tree of other positions: hits equal the
    oracle's on the new positions (camera, bounce and shadow rays, shared
    edges); a refit with the same positions changes nothing; a refit with
    another triangle count is refused."""
    from kiraray_gb300._lib import KrrError
    from kiraray_gb300.accel import set_node_format
    sc = scenes.large_scene(width=160, height=90, grid=256, n_spheres=40, sky_size=(64, 32))
    tris = sc.world_triangles()
    rng = np.random.default_rng(8)
    moved = tris.reshape(-1, 3, 3).copy()
    # a global shear, some triangles moved far (across the tree), all jittered
    moved[..., 0] += 0.15 * moved[..., 1]
    far = rng.choice(moved.shape[0], moved.shape[0] // 50, replace=False)
    moved[far] += rng.normal(0.0, 20.0, (far.size, 1, 3)).astype(np.float32)
    moved += rng.normal(0.0, 1e-3, moved.shape).astype(np.float32)
    moved = moved.reshape(-1, 9).astype(np.float32)
    acc = Accel(tris, node_format=node_format)
    set_node_format(0)
    rays = H.pinhole_rays(sc, jitter_seed=21)
    before = _gpu_closest(acc, rays)
    acc.refit(tris)
    _assert_bits_equal(_gpu_closest(acc, rays), before, "same positions")
    acc.refit(moved)
    ob = O.Bvh(moved)
    want = ob.closest(rays)
    _assert_bits_equal(_gpu_closest(acc, rays), want, "refit camera")
    b = H.bounce_rays(moved, rays, want, 5)
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), "refit bounce")
    assert np.array_equal(acc.trace_any(torch.from_numpy(b).cuda()).cpu().numpy(), ob.any(b))
    g = H.grid_mesh(12)
    r = H.vertex_edge_rays(12, 3)
    ga = Accel(g + 0.5, node_format=node_format)
    set_node_format(0)
    ga.refit(g)
    _assert_bits_equal(_gpu_closest(ga, r), O.closest_brute(g, r), "refit edges")
    with pytest.raises(KrrError):
        acc.refit(moved[:-1])


@pytest.mark.parametrize("leaf,full_leaf", [(1, 1), (2, 2), (3, 3), (1, 2), (1, 3)])
def test_leaf_sizes_keep_hits_identical(krr_lib, cuda, leaf, full_leaf):
    """Leaf children of 1-3 triangles, everywhere or only in full nodes: the
    hits are those of the oracle bit for bit."""
    from kiraray_gb300.accel import set_full_node_leaf, set_max_leaf

    def build(t):
        set_max_leaf(leaf)
        set_full_node_leaf(full_leaf)
        try:
            return Accel(t)
        finally:
            set_max_leaf(1)
            set_full_node_leaf(1)

    sc = scenes.large_scene(width=160, height=90, grid=256, n_spheres=40, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=11)
    acc = build(tris)
    tag = f"leaf {leaf}/{full_leaf}"
    ob = O.Bvh(tris)
    want = ob.closest(rays)
    _assert_bits_equal(_gpu_closest(acc, rays), want, tag)
    b = H.bounce_rays(tris, rays, want, 12)
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), f"{tag} bounce")
    occ = acc.trace_any(torch.from_numpy(b).cuda()).cpu().numpy()
    assert np.array_equal(occ, ob.any(b))
    g = H.grid_mesh(12)
    r = H.vertex_edge_rays(12, 3)
    ga = build(g)
    _assert_bits_equal(_gpu_closest(ga, r), O.closest_brute(g, r), f"{tag} edges")


def test_stack_limit_cuts_rays_off_and_reports_overflow(krr_lib, cuda):
    """A traversal stack limit below the tree's needs cuts rays off: the
    overflow flag is raised, cut-off rays report t = NaN and a miss, every
    other ray keeps its exact hit, and the synchronous entry points return
    KRR_ERR_OVERFLOW.  With the default limit nothing is cut off."""
    from kiraray_gb300._lib import KrrError
    sc = scenes.large_scene(width=96, height=64, grid=128, n_spheres=40, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=2)
    want = O.Bvh(tris).closest(rays)
    acc = Accel(tris)
    assert acc.device_errors() == 0
    acc.set_stack_limit(1)
    got = _gpu_closest(acc, rays)
    assert acc.device_errors() & 1
    cut = np.isnan(got[:, 0])
    assert 0 < cut.sum() < rays.shape[0]
    assert np.all(got[cut, 3].view(np.uint32) == 0xFFFFFFFF)
    _assert_bits_equal(got[~cut], want[~cut], "rays within the stack limit")
    occ = acc.trace_any(torch.from_numpy(rays).cuda()).cpu().numpy()
    assert acc.device_errors() & 1
    assert set(np.unique(occ)) <= {0, 1, 0xFF} and (occ == 0xFF).any()
    with pytest.raises(KrrError, match="stack limit"):
        acc.trace_stats(torch.from_numpy(rays).cuda())
    acc.set_stack_limit(48)
    _assert_bits_equal(_gpu_closest(acc, rays), want, "default stack limit")
    assert acc.device_errors() == 0
    with pytest.raises(KrrError):
        acc.set_stack_limit(49)


@pytest.mark.parametrize("builder", [0, 1])
def test_builders_give_identical_hits(krr_lib, cuda, builder):
    """The radix tree on per-axis cells and PLOC clustering build other trees
    than the default (radix tree on cubic cells) over the same triangles; the
    hits stay bit-identical to the oracle's."""
    from kiraray_gb300.accel import set_builder
    sc = scenes.large_scene(width=160, height=90, grid=256, n_spheres=60, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=9)
    ob = O.Bvh(tris)
    want = ob.closest(rays)
    b = H.bounce_rays(tris, rays, want, 4)
    set_builder(builder)
    try:
        acc = Accel(tris)
        soup = H.random_soup(3000, 17)
        acc_soup = Accel(soup)
        single = Accel(soup[:1])
    finally:
        set_builder(2)
    _assert_bits_equal(_gpu_closest(acc, rays), want, f"builder {builder} camera rays")
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), f"builder {builder} bounce rays")
    r = H.random_rays(2000, 18)
    _assert_bits_equal(_gpu_closest(acc_soup, r), O.closest_brute(soup, r), f"builder {builder} soup")
    _assert_bits_equal(_gpu_closest(single, r), O.closest_brute(soup[:1], r), "one triangle")
    assert acc.stats()["max_depth"] <= 48
    assert acc.device_errors() == 0


@pytest.mark.parametrize("builder", [2, 1, 0])
def test_cost_optimal_collapse_gives_identical_hits(krr_lib, cuda, builder):
    """The cost-optimal collapse cuts the binary tree into other wide nodes
    than the greedy one; hits stay the
    oracle's bit for bit, for scenes, soups, a single triangle and a pile of
    coincident triangles (ties to the smaller id)."""
    from kiraray_gb300.accel import set_builder, set_collapse
    sc = scenes.large_scene(width=160, height=90, grid=256, n_spheres=60, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=21)
    ob = O.Bvh(tris)
    want = ob.closest(rays)
    b = H.bounce_rays(tris, rays, want, 5)
    soup = H.random_soup(3000, 23)
    pile = np.repeat(soup[:1], 700, axis=0)
    set_builder(builder)
    set_collapse(1)
    try:
        acc = Accel(tris)
        acc_soup = Accel(soup)
        single = Accel(soup[:1])
        acc_pile = Accel(pile)
    finally:
        set_builder(2)
        set_collapse(0)
    tag = f"builder {builder}"
    _assert_bits_equal(_gpu_closest(acc, rays), want, f"{tag} camera rays")
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), f"{tag} bounce rays")
    occ = acc.trace_any(torch.from_numpy(b).cuda()).cpu().numpy()
    assert np.array_equal(occ, ob.any(b))
    r = H.random_rays(2000, 24)
    _assert_bits_equal(_gpu_closest(acc_soup, r), O.closest_brute(soup, r), f"{tag} soup")
    _assert_bits_equal(_gpu_closest(single, r), O.closest_brute(soup[:1], r), "one triangle")
    _assert_bits_equal(_gpu_closest(acc_pile, r), O.closest_brute(pile, r), "coincident triangles")
    assert acc.stats()["max_depth"] <= 48
    for a in (acc, acc_soup, single, acc_pile):
        assert a.device_errors() == 0


@pytest.mark.parametrize("builder,passes,collapse", [(2, 1, 0), (2, 3, 0), (1, 2, 0), (0, 1, 1)])
def test_treelet_restructuring_gives_identical_hits(krr_lib, cuda, builder, passes, collapse):
    """Treelet passes rebuild parts of the binary tree before the collapse;
    hits stay the oracle's bit for bit (scene, soup, one triangle, a pile of
    coincident triangles), and the restructured scene tree has other wide
    nodes than the tree as built."""
    from kiraray_gb300._lib import KrrError
    from kiraray_gb300.accel import set_builder, set_collapse, set_treelets
    sc = scenes.large_scene(width=160, height=90, grid=256, n_spheres=60, sky_size=(64, 32))
    tris = sc.world_triangles()
    rays = H.pinhole_rays(sc, jitter_seed=31)
    ob = O.Bvh(tris)
    want = ob.closest(rays)
    b = H.bounce_rays(tris, rays, want, 6)
    soup = H.random_soup(3000, 33)
    pile = np.repeat(soup[:1], 700, axis=0)
    set_builder(builder)
    set_collapse(collapse)
    try:
        plain = Accel(tris)
        set_treelets(passes)
        acc = Accel(tris)
        acc_soup = Accel(soup)
        single = Accel(soup[:1])
        acc_pile = Accel(pile)
    finally:
        set_builder(2)
        set_collapse(0)
        set_treelets(0)
    tag = f"builder {builder}, {passes} treelet passes"
    _assert_bits_equal(_gpu_closest(acc, rays), want, f"{tag} camera rays")
    _assert_bits_equal(_gpu_closest(acc, b), ob.closest(b), f"{tag} bounce rays")
    occ = acc.trace_any(torch.from_numpy(b).cuda()).cpu().numpy()
    assert np.array_equal(occ, ob.any(b))
    r = H.random_rays(2000, 34)
    _assert_bits_equal(_gpu_closest(acc_soup, r), O.closest_brute(soup, r), f"{tag} soup")
    _assert_bits_equal(_gpu_closest(single, r), O.closest_brute(soup[:1], r), "one triangle")
    _assert_bits_equal(_gpu_closest(acc_pile, r), O.closest_brute(pile, r), "coincident triangles")
    assert acc.stats()["n_nodes"] != plain.stats()["n_nodes"]
    assert acc.stats()["max_depth"] <= 48 and acc_pile.stats()["max_depth"] <= 48
    for a in (acc, acc_soup, single, acc_pile):
        assert a.device_errors() == 0
    with pytest.raises(KrrError):
        set_treelets(4)


def test_two_level_structure_matches_the_instanced_oracle(krr_lib, cuda):
    """Geometry trees in object space plus an instance tree: closest hits
    bit-exact against the oracle's two-level restatement (same world-to-object
    matrices), any-hit with per-instance masks, and again after the
    instances move (only the instance level is rebuilt)."""
    from tests.test_oracle import _instanced_scene
    geos, insts = _instanced_scene(seed=5, n_inst=60)
    # an identity instance: its object-space ray is the world ray bit for bit
    insts.append((1, np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)))
    mask = np.ones(len(insts), np.uint8)
    mask[::7] = 0
    acc = Accel.instanced(geos, insts, mask)
    st = acc.stats()
    assert st["n_triangles"] == sum(geos[g].shape[0] for g, _ in insts)
    rays = H.random_rays(20000, 9, box=5.0)
    d_rays = torch.from_numpy(rays).cuda()
    inv = acc.instance_inverse()
    want = O.trace_instanced(geos, insts, inv, rays)
    got = _gpu_closest(acc, rays)
    _assert_bits_equal(got, want, "two-level closest")
    assert (got[:, 3].view(np.uint32) != 0xFFFFFFFF).mean() > 0.05
    occ = acc.trace_any(d_rays).cpu().numpy()
    assert np.array_equal(occ, O.trace_instanced(geos, insts, inv, rays, mask=mask, any_hit=True))
    # move every instance: the instance level is rebuilt, hits follow
    moved = [(g, np.asarray(m, np.float32).copy()) for g, m in insts]
    for k, (g, m) in enumerate(moved):
        m[:, 3] += np.array([0.3 * np.sin(k), 0.2, -0.1 * k / len(moved)], np.float32)
    acc.update_instances(np.stack([m for _, m in moved]))
    inv2 = acc.instance_inverse()
    assert not np.array_equal(inv, inv2)
    _assert_bits_equal(_gpu_closest(acc, rays), O.trace_instanced(geos, moved, inv2, rays),
                       "two-level closest after an update")
    assert acc.device_errors() == 0
    # a stack limit below the two levels' needs cuts rays off (flag raised,
    # t = NaN and a miss); the others keep their exact hits
    want2 = O.trace_instanced(geos, moved, inv2, rays)
    acc.set_stack_limit(3)
    got = _gpu_closest(acc, rays)
    assert acc.device_errors() & 1
    cut = np.isnan(got[:, 0])
    assert 0 < cut.sum() < rays.shape[0]
    assert np.all(got[cut, 3].view(np.uint32) == 0xFFFFFFFF)
    _assert_bits_equal(got[~cut], want2[~cut], "two-level rays within the stack limit")
    acc.set_stack_limit(48)
    _assert_bits_equal(_gpu_closest(acc, rays), want2, "two-level default stack limit")
    assert acc.device_errors() == 0
