"""The offset-fit oracle on its own: an exact affine field is recovered, the
PRM split (ishift, sub_int) truncates toward zero, gross outliers are
discounted by the robust passes, and low-correlation points are left out."""
import numpy as np

import fit_oracle as fo
import xcorr_oracle as xo


def _records(locs, o_r, o_a, corr, ri=2):
    r = np.zeros(len(locs), dtype=xo.RESULT_DTYPE)
    r["xoff"] = (np.asarray(o_r) * ri).astype(np.float32)     # xoff/ri - xfrac/ri = o_r with xfrac 0
    r["yoff"] = np.asarray(o_a, np.float32)
    r["corr"] = corr
    return r


def _grid():
    xs, ys = np.meshgrid(np.arange(300, 1800, 75), np.arange(300, 3800, 70))
    return np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)


def test_exact_affine_field():
    locs = _grid()
    o_r = -7.25 + 3e-4 * locs[:, 0] - 1e-4 * locs[:, 1]
    o_a = 2.5 - 2e-4 * locs[:, 0] + 5e-4 * locs[:, 1]
    f = fo.fit(_records(locs, o_r, o_a, 50.0), locs)
    r, a = f["range"], f["azimuth"]
    assert abs(r["stretch"] - 3e-4) < 1e-8 and abs(r["a_stretch"] + 1e-4) < 1e-8 and abs(r["shift"] + 7.25) < 1e-4
    assert abs(a["stretch"] + 2e-4) < 1e-8 and abs(a["a_stretch"] - 5e-4) < 1e-8 and abs(a["shift"] - 2.5) < 1e-4
    assert r["ishift"] == -7 and abs(r["sub_int"] + 0.25) < 1e-4      # truncation toward zero
    assert a["ishift"] == 2 and abs(a["sub_int"] - 0.5) < 1e-4
    assert r["npts"] == len(locs)


def test_threshold_and_robust_passes():
    rng = np.random.default_rng(3)
    locs = _grid()
    o_r = 1.0 + 2e-4 * locs[:, 0] + rng.normal(0, 0.05, len(locs))
    o_a = -3.0 + 1e-4 * locs[:, 1] + rng.normal(0, 0.05, len(locs))
    bad = rng.choice(len(locs), len(locs) // 20, replace=False)
    o_r[bad] += 25.0
    corr = np.full(len(locs), 40.0, np.float32)
    low = rng.choice(len(locs), 30, replace=False)
    corr[low] = 5.0
    rec = _records(locs, o_r, o_a, corr)
    plain = fo.fit(rec, locs, snr_min=10.0)
    robust = fo.fit(rec, locs, snr_min=10.0, robust_iters=5)
    assert plain["range"]["npts"] == len(locs) - 30
    assert abs(robust["range"]["stretch"] - 2e-4) < 2e-5
    assert abs(robust["range"]["shift"] - 1.0) < 0.05
    assert abs(plain["range"]["shift"] - 1.0) > 0.5          # least squares alone is pulled by the outliers
    assert robust["range"]["rms"] < 0.1
