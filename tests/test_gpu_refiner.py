"""Subpixel refiner kernels on the GPU against the FP64 oracle
(oracle/refiner_oracle.py): forward outputs, loss, every parameter gradient,
one Adam step; the BF16 tensor-core inference against the FP32 forward; and
a few training steps lowering the loss."""
import numpy as np
import pytest

import refiner_oracle as ro
import xcorr_gb300 as xg

pytestmark = pytest.mark.gpu


def _batch(n, seed):
    """Peak-like 9x9 neighbourhoods: a Gaussian bump near the centre plus noise."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:9, 0:9]
    f = np.zeros((n, 81), np.float32)
    t = rng.uniform(-0.5, 0.5, (n, 2)).astype(np.float32)
    for i in range(n):
        w = rng.uniform(0.8, 2.0)
        b = np.exp(-((xx - 4 - t[i, 0]) ** 2 + (yy - 4 - t[i, 1]) ** 2) / (2 * w * w))
        f[i] = (b / b.max() + rng.normal(0, 0.05, b.shape)).ravel()
    return f, t


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def test_gradients_match_fp64_oracle(torch):
    theta = ro.init(7).astype(np.float32)
    f, t = _batch(96, 1)
    ref = xg.Refiner(0, max_batch=128)
    ref.set_params(theta)
    df, dt = torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()
    loss, g, out = ref.gradient(df.data_ptr(), dt.data_ptr(), len(f))
    l64, g64, o64 = ro.loss_grad(theta.astype(np.float64), f, t)
    np.testing.assert_allclose(out, o64, rtol=1e-4, atol=1e-5)
    assert abs(loss - l64) <= 1e-5 * max(1.0, abs(l64))
    rel = np.linalg.norm(g - g64) / np.linalg.norm(g64)
    assert rel < 1e-4, rel
    # every parameter block on its own
    o = 0
    for name, shape in ro.PARAM_LAYOUT:
        k = int(np.prod(shape))
        blk = np.linalg.norm(g[o:o + k] - g64[o:o + k]) / max(np.linalg.norm(g64[o:o + k]), 1e-30)
        assert blk < 1e-3, (name, blk)
        o += k


def test_adam_step_matches_oracle(torch):
    theta = ro.init(3).astype(np.float32)
    f, t = _batch(64, 2)
    ref = xg.Refiner(0, max_batch=64)
    ref.set_params(theta)
    df, dt = torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()
    _, g, _ = ref.gradient(df.data_ptr(), dt.data_ptr(), 64)
    ref.train_step(df.data_ptr(), dt.data_ptr(), 64, 1e-3)
    torch.cuda.synchronize()
    got = ref.get_params()
    want, _, _ = ro.adam(theta.astype(np.float64), g.astype(np.float64), 0.0, 0.0, 1, 1e-3)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-7)


def test_tensor_core_inference_matches_fp32_forward(torch):
    theta = ro.init(11).astype(np.float32)
    f, t = _batch(203, 4)                        # not a multiple of the 4-window groups
    ref = xg.Refiner(0, max_batch=256)
    ref.set_params(theta)
    df = torch.from_numpy(f).cuda()
    o32 = torch.zeros((len(f), 3), device="cuda")
    o16 = torch.zeros((len(f), 3), device="cuda")
    ref.forward(df.data_ptr(), len(f), o32.data_ptr(), tensor_cores=False)
    ref.forward(df.data_ptr(), len(f), o16.data_ptr(), tensor_cores=True)
    torch.cuda.synchronize()
    a, b = o32.cpu().numpy(), o16.cpu().numpy()
    o64, _ = ro.forward(theta.astype(np.float64), f)
    np.testing.assert_allclose(a, o64, rtol=1e-4, atol=1e-5)
    # BF16 weights and activations, FP32 accumulation: about 3 significant digits
    assert np.max(np.abs(b - a)) < 0.05 * max(1.0, np.max(np.abs(a)))
    assert np.sqrt(np.mean((b - a) ** 2)) < 0.01 * max(1.0, np.sqrt(np.mean(a ** 2)))


def test_training_steps_lower_the_loss(torch):
    from xcorr_gb300.refiner_train import init_params
    f, t = _batch(1024, 5)
    ref = xg.Refiner(0, max_batch=1024)
    ref.set_params(init_params(0))
    df, dt = torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()
    l0, _, out0 = ref.gradient(df.data_ptr(), dt.data_ptr(), 1024)
    for _ in range(100):
        ref.train_step(df.data_ptr(), dt.data_ptr(), 1024, 2e-3)
    l1, _, out = ref.gradient(df.data_ptr(), dt.data_ptr(), 1024)
    assert l1 < l0 - 1.0, (l0, l1)
    rms0 = np.sqrt(np.mean((out0[:, :2] - t) ** 2))
    rms1 = np.sqrt(np.mean((out[:, :2] - t) ** 2))
    assert rms1 < 0.8 * rms0, (rms0, rms1)
