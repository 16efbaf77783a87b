"""Cache checkpoints and divergence on the GPU.

- save/load: a fresh cache loaded from a checkpoint holds the same weights,
  hash table, Adam moments and step, answers queries bit for bit like the
  saved one, and its next training step matches the saved cache's next step
  (within the rounding of the atomic gradient sums, whose order varies).
- divergence: a training batch with non-finite targets (injected on the
  host) makes the loss non-finite; the cache marks itself diverged, takes no
  further steps, and a pass with it attached renders exactly the plain
  tracer's frame until new parameters are set."""
import numpy as np
import pytest
import torch

from kiraray_gb300 import scenes
from kiraray_gb300._lib import KrrError
from kiraray_gb300.nrc import NeuralRadianceCache
from kiraray_gb300.wavefront import WavefrontPathTracer
from tests.test_nrc_gpu import SMALL, _records, _rel, _targets

pytestmark = pytest.mark.gpu


def _train(cache, rec, tgt, steps):
    for _ in range(steps):
        cache.train_step(rec, tgt)
    torch.cuda.synchronize()


def test_checkpoint_round_trip(krr_lib, cuda, tmp_path):
    lo, hi = (-1, -1, -1), (1, 1, 1)
    rec = torch.from_numpy(_records(4096, 41)).cuda()
    tgt = torch.from_numpy(_targets(rec.cpu().numpy())).cuda()
    a = NeuralRadianceCache(lo, hi, seed=1, learning_rate=3e-3, **SMALL)
    _train(a, rec, tgt, 7)
    path = tmp_path / "cache.bin"
    a.save(path)
    b = NeuralRadianceCache(lo, hi, seed=2, **SMALL)   # other initial weights and settings
    assert not np.array_equal(a.params(0), b.params(0))
    b.load(path)
    assert b.info().step == a.info().step == 7
    for which in (0, 1):
        assert np.array_equal(a.params(which).view(np.uint32), b.params(which).view(np.uint32))
    q = torch.from_numpy(_records(3000, 42)).cuda()
    qa, qb = a.query(q).cpu().numpy(), b.query(q).cpu().numpy()
    assert np.array_equal(qa.view(np.uint32), qb.view(np.uint32))
    # one more step from the same state: the Adam moments came back too
    fresh = NeuralRadianceCache(lo, hi, seed=2, **SMALL)
    fresh.set_params(0, a.params(0))
    fresh.set_params(1, a.params(1))   # weights only, moments zero
    _train(a, rec, tgt, 1)
    _train(b, rec, tgt, 1)
    _train(fresh, rec, tgt, 1)
    d_ab = _rel(b.params(0), a.params(0))
    d_fresh = _rel(fresh.params(0), a.params(0))
    assert d_ab < 1e-4, d_ab
    assert d_fresh > 10 * d_ab
    assert a.info().step == b.info().step == 8


def test_checkpoint_keeps_the_moving_average(krr_lib, cuda, tmp_path):
    """With a moving average for the queries the checkpoint carries it: the
    loaded cache answers queries bit for bit like the saved one; a cache
    without one loads the same file and queries the trained parameters."""
    lo, hi = (-1, -1, -1), (1, 1, 1)
    rec = torch.from_numpy(_records(4096, 43)).cuda()
    tgt = torch.from_numpy(_targets(rec.cpu().numpy())).cuda()
    a = NeuralRadianceCache(lo, hi, seed=1, ema_decay=0.9, **SMALL)
    _train(a, rec, tgt, 6)
    path = tmp_path / "cache_ema.bin"
    a.save(path)
    b = NeuralRadianceCache(lo, hi, seed=2, ema_decay=0.5, **SMALL)
    b.load(path)
    for which in (0, 1, 2, 3):
        assert np.array_equal(a.params(which).view(np.uint32), b.params(which).view(np.uint32)), which
    q = torch.from_numpy(_records(2000, 44)).cuda()
    assert np.array_equal(a.query(q).cpu().numpy().view(np.uint32), b.query(q).cpu().numpy().view(np.uint32))
    c = NeuralRadianceCache(lo, hi, seed=2, **SMALL)
    c.load(path)
    for which in (0, 1):
        assert np.array_equal(a.params(which).view(np.uint32), c.params(which).view(np.uint32))


def test_checkpoint_rejects_another_shape(krr_lib, cuda, tmp_path):
    a = NeuralRadianceCache((0, 0, 0), (1, 1, 1), **SMALL)
    path = tmp_path / "cache.bin"
    a.save(path)
    other = NeuralRadianceCache((0, 0, 0), (1, 1, 1), n_levels=6, log2_table_size=14,
                                base_resolution=4, max_resolution=64)
    with pytest.raises(KrrError, match="differs"):
        other.load(path)
    (tmp_path / "junk.bin").write_bytes(b"not a checkpoint")
    with pytest.raises(KrrError):
        a.load(tmp_path / "junk.bin")


def test_divergence_falls_back_to_the_plain_tracer(krr_lib, cuda):
    sc = scenes.cornell_box(64, 64, max_depth=5)
    plain = WavefrontPathTracer({"max_depth": 5})
    plain.set_scene(sc)
    plain.resize(64, 64)
    plain.begin_frame(3, sc.camera)
    want = plain.render().cpu().numpy()

    cache = NeuralRadianceCache((0, 0, 0), (1, 1, 1), batch_size=4096, termination_spread=0.0)
    rec = torch.from_numpy(_records(2048, 43)).cuda()
    tgt = torch.from_numpy(_targets(rec.cpu().numpy())).cuda()
    _train(cache, rec, tgt, 3)
    assert cache.status() == (0, False)
    pt = WavefrontPathTracer({"max_depth": 5})
    pt.set_scene(sc)
    pt.resize(64, 64)
    pt.set_nrc(cache, train=True)
    pt.begin_frame(3, sc.camera)
    with_cache = pt.render().cpu().numpy()
    assert not np.array_equal(with_cache, want)   # paths stop at the cache

    bad = tgt.clone()
    bad[17, 1] = float("nan")                     # injected on the host side
    loss = cache.train_step(rec, bad)
    assert not np.isfinite(loss)
    flags, diverged = cache.status()
    assert diverged and flags == 0
    w = cache.params(0)
    step = cache.info().step
    pt.begin_frame(3, sc.camera)
    got = pt.render().cpu().numpy()               # the pass also trains: no step is taken
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert cache.info().step == step
    assert np.array_equal(cache.params(0).view(np.uint32), w.view(np.uint32))
    assert pt.device_errors() == 0
    cache.set_params(0, w)                         # new parameters clear the state
    assert cache.status() == (0, False)
