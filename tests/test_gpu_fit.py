"""xcg_fit_offsets (the fitoffset step on the device) against the float64
numpy oracle: a pair with a known affine shift field is correlated on the
GPU, the fit runs on the device result array, and its coefficients match the
oracle's fit of the same results; the fitted field recovers the synthetic
one."""
import ctypes

import numpy as np
import pytest

import fit_oracle as fo
import xcorr_gb300 as xg
from xcorr_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _pair():
    # piecewise-constant affine field dx = 1.3 + 4e-4 x - 2e-4 y, dy = -2.1 + 1e-4 x + 3e-4 y
    fx = lambda x, y: (1.3 + 4e-4 * x - 2e-4 * y, -2.1 + 1e-4 * x + 3e-4 * y)
    m, s, truth = synth.make_pair_varying(2048, 4096, fx, noise_frac=0.05, seed=5, tile=256, margin=64)
    return m, s, truth


@pytest.fixture(scope="module")
def correlated():
    m, s, truth = _pair()
    p = xg.params(32, 32)
    locs = xg.grid(m.shape[1], m.shape[0], 24, 40, 32, 32)
    dev = torch.device("cuda")
    dm = torch.from_numpy(m.view(np.int32).reshape(m.shape[0], m.shape[1])).to(dev)
    ds = torch.from_numpy(s.view(np.int32).reshape(s.shape[0], s.shape[1])).to(dev)
    dl = torch.from_numpy(locs.reshape(-1)).to(dev)
    dr = torch.zeros(len(locs) * xg.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    with xg.Context(p) as ctx:
        ctx.correlate_device(dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1], s.shape[0],
                             dl.data_ptr(), len(locs), dr.data_ptr(), strip_len=24)
    torch.cuda.synchronize()
    res = np.frombuffer(dr.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)
    return locs, dl, dr, res, truth


def _gpu_fit(dl, dr, n, **kw):
    out = torch.zeros(ctypes.sizeof(xg.Fit), dtype=torch.uint8, device="cuda")
    xg.fit_offsets(dr.data_ptr(), dl.data_ptr(), n, out.data_ptr(), **kw)
    torch.cuda.synchronize()
    return xg.Fit.from_buffer_copy(out.cpu().numpy().tobytes())


@pytest.mark.parametrize("npar,robust", [(3, 0), (2, 0), (1, 0), (3, 3)])
def test_fit_matches_oracle(correlated, npar, robust):
    locs, dl, dr, res, _ = correlated
    f = _gpu_fit(dl, dr, len(locs), snr_min=10.0, npar_range=npar, npar_azimuth=npar, robust_iters=robust)
    o = fo.fit(res, locs, snr_min=10.0, npar_range=npar, npar_azimuth=npar, robust_iters=robust)
    for axis in ("range", "azimuth"):
        g, r = getattr(f, axis), o[axis]
        assert g.npts == r["npts"] > 0.9 * len(locs)
        assert g.ishift == r["ishift"]
        for k in ("shift", "stretch", "a_stretch", "rms", "weight"):
            assert abs(getattr(g, k) - r[k]) <= 1e-9 * max(1.0, abs(r[k])), (axis, k, getattr(g, k), r[k])


def test_fit_recovers_the_shift_field(correlated):
    locs, dl, dr, res, _ = correlated
    f = _gpu_fit(dl, dr, len(locs), snr_min=10.0, robust_iters=3)
    # the slave is the master delayed by the field, so offsets = field (range, azimuth);
    # the field is constant per 256-pixel tile and azimuth offsets carry the
    # estimator's pixel-locking bias (no azimuth oversampling), hence the margins
    assert abs(f.range.stretch - 4e-4) < 3e-5 and abs(f.range.a_stretch + 2e-4) < 3e-5
    assert abs(f.azimuth.stretch - 1e-4) < 6e-5 and abs(f.azimuth.a_stretch - 3e-4) < 6e-5
    assert abs(f.range.shift - 1.3) < 0.1 and abs(f.azimuth.shift + 2.1) < 0.15


def test_fit_rejects_bad_arguments(correlated):
    locs, dl, dr, res, _ = correlated
    with pytest.raises(xg.XcgError):
        _gpu_fit(dl, dr, len(locs), npar_range=4)
