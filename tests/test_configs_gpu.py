"""Parity at the benchmark configurations' own sizes (GPU against the CPU
restatement), rather than at the reduced sizes of the other frame tests.

- Cornell box, 512x512, max depth 5, seed 0: every pixel of two frames.
- Large scene, 10.9M triangles (2048x2048 heightfield + 500 icospheres),
  1920x1080, max depth 8, seed 1: the GPU renders the whole frame; two bands
  of rows are compared with the oracle (the oracle's BVH is built once).
- Volume box, 256^3 FP16 density with a 16^3 majorant grid, 1024x1024,
  max depth 16, seed 2: every pixel.
- Neural radiance cache with the benchmark's hash configuration (16 levels,
  2^19 entries per level, resolutions 16..2048): predictions and gradients
  against the numpy oracle, with hash collisions on the fine levels.

Per-pixel tolerance as tests/test_wavefront_gpu.py; the frames also bound
how far the outlier pixels are off (`compare`).  The 1080p large scene allows
0.5 % outlier pixels instead of 0.2 %: its GGX conductors and dielectrics go
down to roughness 0.05 (alpha 0.0025), and we attribute the outliers to
those narrow lobes turning the 1-2 ulp differences of CUDA's and glibc's
sinf/cosf/acosf/atan2f into relative radiance differences of 1e-4 to 1e-3
on about 0.3 % of the pixels; the frame-level bounds stay as tight as
elsewhere."""
import numpy as np
import pytest
import torch

from kiraray_gb300 import scenes
from kiraray_gb300.nrc import NeuralRadianceCache
from kiraray_gb300.wavefront import WavefrontPathTracer
from oracle import nrc_ref as R
from oracle import pyoracle as O
from tests.test_nrc_gpu import _oracle, _records, _rel, _targets
from tests.test_wavefront_gpu import compare, gpu_frame

pytestmark = pytest.mark.gpu

CONFIG3 = dict(n_levels=16, log2_table_size=19, base_resolution=16, max_resolution=2048)


def _pass(sc):
    pt = WavefrontPathTracer({"max_depth": sc.max_depth}, seed=0)
    pt.set_scene(sc)
    pt.resize(sc.width, sc.height)
    return pt


@pytest.mark.parametrize("frame", [1, 2])
def test_config0_cornell_box_512_every_pixel(krr_lib, cuda, frame):
    sc = scenes.cornell_box(512, 512, max_depth=5, seed=0)
    pt = _pass(sc)
    L, img = gpu_frame(pt, sc, frame)
    oL, opx = O.PathTracer(sc).render({"max_depth": 5}, frame)
    compare(L[:, :3], oL, f"cornell 512 frame {frame}")
    want = opx.reshape(512, 512, 3)[::-1]
    compare(img[..., :3].reshape(-1, 3), want.reshape(-1, 3), f"cornell 512 output {frame}")
    assert pt.device_errors() == 0


@pytest.mark.slow
def test_config1_large_scene_1080p_row_bands(krr_lib, cuda):
    sc = scenes.large_scene()   # 1920x1080, max depth 8, seed 1, 10.9M triangles
    assert sc.n_triangles > 10_000_000
    pt = _pass(sc)
    L, _ = gpu_frame(pt, sc, 1)
    assert pt.device_errors() == 0
    ora = O.PathTracer(sc)
    w = sc.width
    for r0, r1 in ((300, 340), (700, 740)):   # terrain and spheres; foreground terrain
        oL, _ = ora.render({"max_depth": 8}, 1, r0 * w, r1 * w)
        compare(L[r0 * w:r1 * w, :3], oL, f"1080p rows {r0}..{r1}", max_outliers=0.005)
        assert (oL.sum(1) > 0).mean() > 0.3


@pytest.mark.slow
def test_config2_volume_box_1024_every_pixel(krr_lib, cuda):
    sc = scenes.volume_box(1024, 1024, max_depth=16, seed=2)   # 256^3 grid, 16^3 majorant
    pt = _pass(sc)
    L, img = gpu_frame(pt, sc, 1)
    assert pt.device_errors() == 0
    oL, _ = O.PathTracer(sc).render({"max_depth": 16}, 1)
    compare(L[:, :3], oL, "volume 1024")
    assert np.isfinite(img).all()


def _config3_cache(seed):
    lo, hi = (-1, -1, -1), (1, 1, 1)
    cache = NeuralRadianceCache(lo, hi, **CONFIG3)
    info = cache.info()
    assert info.n_levels == 16 and info.resolution[15] == 2048
    assert max(info.level_size[:16]) == 1 << 19
    rec = _records(8192, seed)
    for _ in range(10):
        cache.train_step(torch.from_numpy(rec).cuda(), torch.from_numpy(_targets(rec)).cuda())
    return cache, lo, hi


def test_config3_hash_grid_forward_matches_oracle(krr_lib, cuda):
    cache, lo, hi = _config3_cache(31)
    rec = _records(20000, 32)
    got = cache.query(torch.from_numpy(rec).cuda()).cpu().numpy()
    grid, mlp, table, _ = _oracle(cache, lo, hi)
    X0, _ = R.encode(grid, table, rec)
    want, _ = R.forward(mlp, X0)
    assert _rel(got, want) < 2e-2
    assert np.median(np.abs(got - want) / (np.abs(want) + 1e-3)) < 5e-3


def test_config3_hash_grid_gradients_match_oracle(krr_lib, cuda):
    cache, lo, hi = _config3_cache(33)
    rec = _records(16384, 34)
    tgt = _targets(rec)
    gm, gt, loss = cache.gradients(torch.from_numpy(rec).cuda(), torch.from_numpy(tgt).cuda())
    grid, mlp, table, info = _oracle(cache, lo, hi)
    X0, cs = R.encode(grid, table, rec)
    y, acts = R.forward(mlp, X0)
    want_loss, dy = R.loss_and_grad(y, tgt.astype(np.float64))
    gW, dX0 = R.backward(mlp, acts, dy, loss_scale=cache.cfg.loss_scale)
    gT = R.table_grad(grid, cs, dX0, info.n_table_entries)
    assert abs(loss - want_loss) < 1e-2 * want_loss
    o = 0
    for layer in range(mlp.layers):
        rows = R.WIDTH if layer + 1 < mlp.layers else R.OUT_PAD
        g = gm[o:o + rows * R.IN].reshape(rows, R.IN)
        o += rows * R.IN
        assert _rel(g, gW[layer]) < 3e-2, f"layer {layer}"
    assert _rel(gt, gT) < 3e-2
    # the fine levels are hashed: several records share entries there
    fine = slice(int(info.level_offset[15]) * 2, (int(info.level_offset[15]) + (1 << 19)) * 2)
    assert np.count_nonzero(gT[fine]) > 0
