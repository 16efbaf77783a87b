"""FP64 accumulation and relMSE/MSE on the GPU against numpy float64."""
import numpy as np
import pytest
import torch

from kiraray_gb300.convergence import MSE, RELMSE, Accumulator

pytestmark = pytest.mark.gpu


def _numpy_error(mean_rgb, ref_rgb, metric):
    d = np.abs(mean_rgb - ref_rgb)
    if metric == RELMSE:
        with np.errstate(divide="ignore", invalid="ignore"):
            e = np.where(ref_rgb == 0, 0.0, (d / ref_rgb) ** 2)
    else:
        e = d ** 2
    return np.minimum(e.mean(1), 100.0).mean()


@pytest.mark.parametrize("metric", [RELMSE, MSE])
def test_accumulate_and_error(krr_lib, cuda, metric):
    rng = np.random.default_rng(3)
    n = 50000
    ref = np.ones((n, 4), np.float32)
    ref[:, :3] = rng.random((n, 3)).astype(np.float32)
    ref[::7, 1] = 0.0                       # zero reference channels contribute 0
    frames = [rng.random((n, 4)).astype(np.float32) * 2 for _ in range(5)]
    frames[2][::11, 0] = 1e6                # outliers are clamped at 100 per pixel
    acc = Accumulator(n, 1)
    for f in frames:
        acc.add(torch.from_numpy(f).cuda())
    got = acc.error(torch.from_numpy(ref).cuda(), metric)
    mean = np.sum([f[:, :3].astype(np.float64) for f in frames], 0) / 5
    want = _numpy_error(mean, ref[:, :3].astype(np.float64), metric)
    assert abs(got - want) <= 1e-12 * max(1.0, abs(want))
    assert np.allclose(acc.sum.cpu().numpy(), np.sum([f[:, :3].astype(np.float64) for f in frames], 0))


@pytest.mark.parametrize("op", range(5))
@pytest.mark.parametrize("gamma", [False, True])
def test_tonemap_matches_oracle(krr_lib, cuda, op, gamma):
    from kiraray_gb300.convergence import TONEMAP_OPERATORS, tonemap
    from oracle.imagepasses import tonemap as tonemap_ref
    rng = np.random.default_rng(op)
    img = np.zeros((37, 53, 4), np.float32)
    img[..., :3] = rng.exponential(0.8, (37, 53, 3)).astype(np.float32)
    img[0, :5, :3] = 0.0          # black pixels (Reinhard's 0/0 guard)
    got = tonemap(torch.from_numpy(img).cuda(), TONEMAP_OPERATORS[op], 1.7, gamma).cpu().numpy()
    want = tonemap_ref(img, op, 1.7, gamma)
    assert np.all(got[..., 3] == 1.0)
    np.testing.assert_allclose(got, want, rtol=2e-6, atol=2e-7)


def test_accumulation_checkpoint_resumes(krr_lib, cuda, tmp_path):
    """An FP64 accumulation saved after some frames and loaded into a new
    accumulator continues to the same sum bit for bit."""
    frames = [torch.rand((32 * 16, 4), device="cuda") for _ in range(6)]
    a = Accumulator(32, 16)
    for f in frames[:4]:
        a.add(f)
    a.save(tmp_path / "acc.bin")
    b = Accumulator(32, 16)
    b.load(tmp_path / "acc.bin")
    for f in frames[4:]:
        a.add(f)
        b.add(f)
    assert b.frames == a.frames == 6
    assert torch.equal(a.sum, b.sum)
    with pytest.raises(ValueError):
        Accumulator(8, 8).load(tmp_path / "acc.bin")
