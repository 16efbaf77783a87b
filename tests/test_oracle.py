"""CPU checks of the oracle against known answers (no GPU)."""
import numpy as np
import pytest

from kiraray_gb300 import scenes
from oracle import pyoracle as O
from tests import helpers as H


def test_pcg32_published_vector(oracle_lib):
    # Output of the published pcg32 demo (pcg-random.org, minimal C library)
    # seeded with initstate 42, initseq 54.  The reference's PCGSampler seeds
    # the same way (src/core/sampler.h:22-28).
    got = O.pcg_u32(42, 54, 6)
    want = [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]
    assert [int(x) for x in got] == want


def test_interleave_32bit(oracle_lib):
    assert oracle_lib.oracle_interleave_32bit(0xFFFF, 0) == 0x55555555
    assert oracle_lib.oracle_interleave_32bit(0, 0xFFFF) == 0xAAAAAAAA
    assert oracle_lib.oracle_interleave_32bit(3, 1) == 0b111
    # only the low 16 bits of each coordinate count (src/util/hash.h:13-14)
    assert oracle_lib.oracle_interleave_32bit(0x10000, 0x10000) == 0


def test_pcg_advance_equals_stepping(oracle_lib):
    base = O.pcg_floats(17, 5, 3, 0, 300)
    for k in (1, 2, 7, 64, 256):
        adv = O.pcg_floats(17, 5, 3, k, 10)
        assert np.array_equal(adv, base[k:k + 10])


def test_pcg_floats_in_unit_interval(oracle_lib):
    f = O.pcg_floats(1, 2, 3, 1000, 100000)
    assert f.min() >= 0.0 and f.max() < 1.0
    assert abs(f.mean() - 0.5) < 0.01


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_bvh_equals_brute_force(oracle_lib, seed):
    tris = H.random_soup(3000, seed)
    rays = H.random_rays(4000, seed + 100)
    brute = O.closest_brute(tris, rays)
    bvh = O.Bvh(tris).closest(rays)
    assert np.array_equal(brute.view(np.uint32), bvh.view(np.uint32))
    assert (brute[:, 3].view(np.uint32) != 0xFFFFFFFF).mean() > 0.2


def test_watertight_grid_vertices_and_edges(oracle_lib):
    tris = H.grid_mesh(12)
    rays = H.vertex_edge_rays(12, 3)
    hits = O.closest_brute(tris, rays)
    assert np.all(hits[:, 3].view(np.uint32) != 0xFFFFFFFF), "ray leaked through a shared edge"
    bvh = O.Bvh(tris).closest(rays)
    assert np.array_equal(hits.view(np.uint32), bvh.view(np.uint32))


def test_watertight_closed_icosphere(oracle_lib):
    m = scenes.icosphere(3)
    tris = m.positions[m.indices].reshape(-1, 9).astype(np.float32)
    rays = H.random_rays(20000, 9, box=0.0)   # all from the centre
    # add rays aimed exactly at vertices from the centre
    vr = np.zeros((m.positions.shape[0], 8), np.float32)
    vr[:, 4:7] = m.positions
    vr[:, 7] = np.inf
    rays = np.concatenate([rays, vr])
    hits = O.Bvh(tris).closest(rays)
    assert np.all(hits[:, 3].view(np.uint32) != 0xFFFFFFFF)


def test_tie_goes_to_smaller_id(oracle_lib):
    t = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    tris = np.concatenate([t, t, t])
    rays = np.array([[0.2, 0.2, 1, 0, 0, 0, -1, np.inf]], np.float32)
    h = O.closest_brute(tris, rays)
    assert h[0, 3].view(np.uint32) == 0
    assert O.Bvh(tris).closest(rays)[0, 3].view(np.uint32) == 0


def test_tmin_tmax_window(oracle_lib):
    t = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0], [0, 0, -1, 1, 0, -1, 0, 1, -1]], np.float32)
    rays = np.array([[0.2, 0.2, 1, 0, 0, 0, -1, np.inf],
                     [0.2, 0.2, 1, 1.5, 0, 0, -1, np.inf],
                     [0.2, 0.2, 1, 0, 0, 0, -1, 0.5]], np.float32)
    h = O.closest_brute(t, rays)
    assert list(h[:, 3].view(np.uint32)) == [0, 1, 0xFFFFFFFF]
    assert np.allclose(h[:2, 0], [1.0, 2.0])


def test_any_hit_mask(oracle_lib):
    tris = H.random_soup(500, 4)
    rays = H.random_rays(2000, 5)
    b = O.Bvh(tris)
    occ = b.any(rays)
    hits = b.closest(rays)
    assert np.array_equal(occ.astype(bool), hits[:, 3].view(np.uint32) != 0xFFFFFFFF)
    b.set_mask(np.zeros(500, np.uint8))
    assert not b.any(rays).any()


def _instanced_scene(seed=3, n_inst=40):
    """Two geometries (an icosphere and a random soup) drawn by rotated,
    scaled and translated instances."""
    from kiraray_gb300 import scenes
    rng = np.random.default_rng(seed)
    sph = scenes.icosphere(2)
    geo0 = sph.positions[sph.indices].reshape(-1, 9).astype(np.float32)
    geo1 = (rng.random((50, 1, 3)) * 0.6 - 0.3 + (rng.random((50, 3, 3)) - 0.5) * 0.2)
    geo1 = geo1.reshape(-1, 9).astype(np.float32)
    insts = []
    for i in range(n_inst):
        a = rng.uniform(0, 2 * np.pi)
        c, s = np.cos(a), np.sin(a)
        k = rng.uniform(0.3, 1.2)
        m = np.array([[c * k, 0, s * k, rng.uniform(-4, 4)], [0, k, 0, rng.uniform(-1, 1)],
                      [-s * k, 0, c * k, rng.uniform(-4, 4)]], np.float32)
        insts.append((i % 2, m))
    return [geo0, geo1], insts


def _inverse(insts):
    out = []
    for _, m in insts:
        full = np.eye(4)
        full[:3] = np.asarray(m, np.float64)
        out.append(np.linalg.inv(full)[:3].astype(np.float32).reshape(12))
    return np.array(out, np.float32)


def test_instanced_oracle_agrees_with_the_flattened_scene():
    """The two-level restatement (object-space rays) finds the same triangles
    as the world-space one on the flattened instances, with t equal up to
    rounding."""
    geos, insts = _instanced_scene()
    flat = []
    for g, m in insts:
        v = geos[g].reshape(-1, 3).astype(np.float64)
        w = v @ np.asarray(m, np.float64)[:, :3].T + np.asarray(m, np.float64)[:, 3]
        flat.append(w.astype(np.float32).reshape(-1, 9))
    flat = np.concatenate(flat)
    rays = H.random_rays(4000, 8, box=5.0)
    want = O.Bvh(flat).closest(rays)
    got = O.trace_instanced(geos, insts, _inverse(insts), rays)
    same = got[:, 3].view(np.uint32) == want[:, 3].view(np.uint32)
    assert same.mean() > 0.995
    hit = same & (want[:, 3].view(np.uint32) != 0xFFFFFFFF)
    assert hit.sum() > 500
    assert np.allclose(got[hit, 0], want[hit, 0], rtol=1e-4)
    occ = O.trace_instanced(geos, insts, _inverse(insts), rays, any_hit=True)
    assert np.array_equal(occ.astype(bool), want[:, 3].view(np.uint32) != 0xFFFFFFFF)
