"""Neural radiance cache on the GPU: predictions and gradients against the
numpy restatement (same BF16 rounding points), training, and the cache in
the wavefront pass."""
import numpy as np
import pytest
import torch

from kiraray_gb300 import scenes
from kiraray_gb300.nrc import NeuralRadianceCache
from kiraray_gb300.wavefront import WavefrontPathTracer
from oracle import nrc_ref as R

pytestmark = pytest.mark.gpu

SMALL = dict(n_levels=8, log2_table_size=14, base_resolution=4, max_resolution=128)


def _records(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 13), np.float32)
    r[:, :3] = rng.random((n, 3)) * 2 - 1
    nrm = rng.normal(size=(n, 3))
    r[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    r[:, 6] = rng.random(n)
    r[:, 7:10] = rng.random((n, 3))
    wo = rng.normal(size=(n, 3))
    r[:, 10:13] = wo / np.linalg.norm(wo, axis=1, keepdims=True)
    return r


def _targets(rec):
    p = rec[:, :3].astype(np.float64)
    return np.stack([1 + np.sin(3 * p[:, 0]), 1 + np.cos(2 * p[:, 1]) * p[:, 2],
                     0.5 + rec[:, 7]], 1).astype(np.float32)


def _oracle(cache, lo, hi):
    info = cache.info()
    grid = R.Grid(info, lo, hi, 1 << cache.cfg.log2_table_size)
    mlp = R.Mlp(cache.params(0).astype(np.float64), cache.cfg.hidden_layers + 1)
    return grid, mlp, cache.params(1).astype(np.float64), info


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def test_moving_average_for_queries(krr_lib, cuda):
    """ema_decay d: after each Adam step the queries' copy of the parameters
    becomes d e + (1 - d) w, and queries read that copy (the oracle's forward
    on it), while training keeps reading the parameters themselves."""
    lo, hi = (-1, -1, -1), (1, 1, 1)
    cache = NeuralRadianceCache(lo, hi, ema_decay=0.75, **SMALL)
    rec = _records(3000, 5)
    r, t = torch.from_numpy(rec).cuda(), torch.from_numpy(_targets(rec)).cuda()
    for which in (0, 1):
        assert np.array_equal(cache.params(which), cache.params(which + 2))
    e = [cache.params(0).astype(np.float64), cache.params(1).astype(np.float64)]
    for s in range(12):
        cache.train_step(r, t)
        for which in (0, 1):
            w = cache.params(which).astype(np.float64)
            e[which] = 0.75 * e[which] + 0.25 * w
            got = cache.params(which + 2)
            assert np.allclose(got, e[which], rtol=1e-5, atol=1e-8), (s, which)
    got = cache.query(r).cpu().numpy()
    info = cache.info()
    grid = R.Grid(info, lo, hi, 1 << cache.cfg.log2_table_size)
    mlp = R.Mlp(cache.params(2).astype(np.float64), cache.cfg.hidden_layers + 1)
    X0, _ = R.encode(grid, cache.params(3).astype(np.float64), rec)
    want, _ = R.forward(mlp, X0)
    assert _rel(got, want) < 2e-2
    # the average lags the trained parameters: their forward differs
    mlp_w = R.Mlp(cache.params(0).astype(np.float64), cache.cfg.hidden_layers + 1)
    X0w, _ = R.encode(grid, cache.params(1).astype(np.float64), rec)
    trained, _ = R.forward(mlp_w, X0w)
    assert _rel(got, trained) > 1.5 * _rel(got, want)
    # set_params restarts the average from the new values
    cache.set_params(0, cache.params(0))
    assert np.array_equal(cache.params(0), cache.params(2))
    plain = NeuralRadianceCache(lo, hi, **SMALL)
    with pytest.raises(Exception):
        plain.params(2)


def test_forward_matches_oracle(krr_lib, cuda):
    lo, hi = (-1, -1, -1), (1, 1, 1)
    cache = NeuralRadianceCache(lo, hi, **SMALL)
    rec = _records(3000, 1)
    # train a few steps so that the prediction is not near zero
    for s in range(20):
        cache.train_step(torch.from_numpy(rec).cuda(), torch.from_numpy(_targets(rec)).cuda())
    got = cache.query(torch.from_numpy(rec).cuda()).cpu().numpy()
    grid, mlp, table, _ = _oracle(cache, lo, hi)
    X0, _ = R.encode(grid, table, rec)
    want, _ = R.forward(mlp, X0)
    assert _rel(got, want) < 2e-2
    assert np.median(np.abs(got - want) / (np.abs(want) + 1e-3)) < 5e-3


def test_gradients_match_oracle(krr_lib, cuda):
    lo, hi = (-1, -1, -1), (1, 1, 1)
    cache = NeuralRadianceCache(lo, hi, **SMALL)
    rec = _records(4096, 2)
    tgt = _targets(rec)
    for s in range(5):
        cache.train_step(torch.from_numpy(rec).cuda(), torch.from_numpy(tgt).cuda())
    gm, gt, loss = cache.gradients(torch.from_numpy(rec).cuda(), torch.from_numpy(tgt).cuda())
    grid, mlp, table, info = _oracle(cache, lo, hi)
    X0, cs = R.encode(grid, table, rec)
    y, acts = R.forward(mlp, X0)
    want_loss, dy = R.loss_and_grad(y, tgt.astype(np.float64))
    gW, dX0 = R.backward(mlp, acts, dy, loss_scale=cache.cfg.loss_scale)
    gT = R.table_grad(grid, cs, dX0, info.n_table_entries)
    assert abs(loss - want_loss) < 1e-2 * want_loss
    o = 0
    for l in range(mlp.layers):
        rows = R.WIDTH if l + 1 < mlp.layers else R.OUT_PAD
        g = gm[o:o + rows * R.IN].reshape(rows, R.IN)
        o += rows * R.IN
        assert _rel(g, gW[l]) < 3e-2, f"layer {l}"
    assert _rel(gt, gT) < 3e-2


def test_tensor_core_forward_matches_cuda_core_kernels(krr_lib, cuda):
    """tcgen05 BF16 MMAs (FP32 accumulation in tensor memory) against the
    CUDA-core kernels with the same BF16 rounding points."""
    lo, hi = (-1, -1, -1), (1, 1, 1)
    tc = NeuralRadianceCache(lo, hi, tensor_cores=1, **SMALL)
    ref = NeuralRadianceCache(lo, hi, tensor_cores=0, **SMALL)
    rec = _records(10000, 5)
    for _ in range(30):
        tc.train_step(torch.from_numpy(rec[:4096]).cuda(),
                      torch.from_numpy(_targets(rec[:4096])).cuda())
    ref.set_params(0, tc.params(0))
    ref.set_params(1, tc.params(1))
    q = torch.from_numpy(rec).cuda()
    a = tc.query(q).cpu().numpy()
    b = ref.query(q).cpu().numpy()
    assert np.isfinite(a).all()
    assert _rel(a, b) < 1e-2
    assert np.median(np.abs(a - b) / (np.abs(b) + 1e-3)) < 2e-3
    # tile edges: counts that are not multiples of 128 rows
    for n in (1, 127, 129, 1000):
        aa = tc.query(q[:n].contiguous()).cpu().numpy()
        assert np.allclose(aa, a[:n], rtol=0, atol=1e-6)


def test_training_reduces_loss(krr_lib, cuda):
    cache = NeuralRadianceCache((-1, -1, -1), (1, 1, 1), **SMALL)
    rec = torch.from_numpy(_records(16384, 3)).cuda()
    tgt = torch.from_numpy(_targets(rec.cpu().numpy())).cuda()
    losses = [cache.train_step(rec, tgt) for _ in range(300)]
    assert np.isfinite(losses).all()
    assert np.mean(losses[-10:]) < 0.1 * np.mean(losses[:3])


def test_cache_in_the_pass(krr_lib, cuda):
    sc = scenes.cornell_box(96, 96, max_depth=5)
    lo, hi = (0, 0, 0), (1, 1, 1)
    plain = WavefrontPathTracer({"max_depth": 5})
    plain.set_scene(sc)
    plain.resize(96, 96)
    pt = WavefrontPathTracer({"max_depth": 5})
    pt.set_scene(sc)
    pt.resize(96, 96)
    cache = NeuralRadianceCache(lo, hi, batch_size=8192)
    pt.set_nrc(cache, train=True)
    acc_p = torch.zeros((96, 96, 4), device="cuda")
    acc_n = torch.zeros((96, 96, 4), device="cuda")
    for f in range(1, 121):
        plain.begin_frame(f, sc.camera)
        acc_p += plain.render()
        pt.begin_frame(f, sc.camera)
        img = pt.render()
        if f > 60:
            acc_n += img
    assert pt.device_errors() == 0
    assert cache.info().step == 120
    mp = (acc_p / 120)[..., :3].mean().item()
    mn = (acc_n / 60)[..., :3].mean().item()
    assert torch.isfinite(acc_n).all()
    assert abs(mn - mp) < 0.15 * mp, (mn, mp)


def test_spread_threshold_controls_termination(krr_lib, cuda):
    """With an unreachable spread threshold no path stops at the cache, so the
    pass draws the same samples as the plain tracer and the frame is equal
    bit for bit; with threshold 0 paths stop at their first rough vertex."""
    sc = scenes.cornell_box(48, 48, max_depth=5)
    plain = WavefrontPathTracer({"max_depth": 5})
    plain.set_scene(sc)
    plain.resize(48, 48)
    plain.begin_frame(3, sc.camera)
    want = plain.render().cpu().numpy()
    imgs = {}
    for c in (1e30, 0.0):
        pt = WavefrontPathTracer({"max_depth": 5})
        pt.set_scene(sc)
        pt.resize(48, 48)
        cache = NeuralRadianceCache((0, 0, 0), (1, 1, 1), batch_size=4096, termination_spread=c)
        pt.set_nrc(cache, train=False)
        pt.begin_frame(3, sc.camera)
        imgs[c] = pt.render().cpu().numpy()
        assert pt.device_errors() == 0
    assert np.array_equal(imgs[1e30].view(np.uint32), want.view(np.uint32))
    assert not np.array_equal(imgs[0.0], want)


def test_cache_queries_of_a_sample_evaluated_at_its_end(krr_lib, cuda):
    """render() evaluates the cache once per sample for the paths that stopped
    at it at any depth; the stage-by-stage loop evaluates it after each
    closest-hit stage.  A stopped path gets no radiance afterwards, so the
    two are equal bit for bit (with a spread threshold of 0, most paths stop
    at their first rough vertex)."""
    sc = scenes.cornell_box(64, 48, max_depth=5)
    cache = NeuralRadianceCache((0, 0, 0), (1, 1, 1), batch_size=4096, termination_spread=0.0, seed=5)
    rec = _records(4096, 3)
    for _ in range(5):   # weights away from their initial values
        cache.train_step(torch.from_numpy(rec).cuda(), torch.from_numpy(_targets(rec)).cuda())
    pt = WavefrontPathTracer({"max_depth": 5}, seed=6)
    pt.set_scene(sc)
    pt.resize(64, 48)
    pt.set_nrc(cache, train=False)
    pt.begin_frame(4, sc.camera)
    pt.render()
    fused = pt.radiance().cpu().numpy()
    pt.begin_frame(4, sc.camera)
    pt.reset_queues(-1)
    pt.generate_camera_rays()
    for d in range(6):
        pt.reset_queues(d)
        pt.trace_closest(d)
        pt.handle_hit()
        pt.handle_miss()
        if d == 5:
            break
        pt.generate_scatter_rays(d)
        pt.trace_shadow()
    staged = pt.radiance().cpu().numpy()
    assert np.array_equal(fused.view(np.uint32), staged.view(np.uint32))
    assert pt.device_errors() == 0


@pytest.mark.parametrize("n", [1, 100, 128, 1000, 4096])
def test_tensor_core_backward_matches_cuda_core_kernels(krr_lib, cuda, n):
    """tcgen05 backward (dX chain and per-layer dW accumulated in tensor
    memory) against the CUDA-core kernels with the same BF16 operands."""
    lo, hi = (-1, -1, -1), (1, 1, 1)
    tc = NeuralRadianceCache(lo, hi, tensor_cores=1, **SMALL)
    ref = NeuralRadianceCache(lo, hi, tensor_cores=0, **SMALL)
    rec = _records(4096, 8)
    for _ in range(10):
        tc.train_step(torch.from_numpy(rec).cuda(), torch.from_numpy(_targets(rec)).cuda())
    ref.set_params(0, tc.params(0))
    ref.set_params(1, tc.params(1))
    q = torch.from_numpy(rec[:n]).cuda()
    t = torch.from_numpy(_targets(rec[:n])).cuda()
    gm_a, gt_a, la = tc.gradients(q, t)
    gm_b, gt_b, lb = ref.gradients(q, t)
    assert np.isfinite(gm_a).all() and np.isfinite(gt_a).all()
    assert abs(la - lb) <= 5e-3 * abs(lb) + 1e-7
    assert _rel(gm_a, gm_b) < 2e-2
    assert _rel(gt_a, gt_b) < 2e-2
    assert tc.info().step == 10
