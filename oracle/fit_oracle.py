"""Oracle for xcg_fit_offsets (test infrastructure only).

A numpy restatement, in float64, of the affine offset fit the library runs on
the device: the step GMTSAR's fitoffset.csh performs on freq_xcorr.dat
(named at xcorr.cu:52; the script is not in the reference sources).  Offsets
are formed as print_results.c:37-38 forms them (float32 arithmetic); points
with corr <= snr_min or non-finite offsets are left out; coordinates are
centred and scaled to [-1, 1]; each axis is fitted by least squares to
c0 + c1*u + c2*v (npar 3), c0 + c1*u (2) or c0 (1), optionally followed by
Tukey-biweight reweighted passes (c = 4.685 times the weighted rms residual
of the previous pass).  Only tests/ import this module, as the checker.
"""
from __future__ import annotations

import numpy as np


def offsets(res, locs, ri, x_offset, y_offset, astretcha):
    f = np.float32
    ishft = np.trunc(locs[:, 1].astype(np.float64) * astretcha).astype(np.int32)
    o_r = (res["xoff"].astype(f) / f(ri)) - (res["xfrac"].astype(f) / f(ri)) + f(x_offset)
    o_a = res["yoff"].astype(f) - res["yfrac"].astype(f) + f(y_offset) + ishft.astype(f)
    return o_r.astype(f), o_a.astype(f)


def fit(res, locs, ri=2, x_offset=0, y_offset=0, astretcha=0.0, snr_min=20.0, npar_range=3, npar_azimuth=3,
        robust_iters=0):
    locs = np.asarray(locs, np.int32).reshape(-1, 2)
    o_r, o_a = offsets(res, locs, ri, x_offset, y_offset, astretcha)
    use = (res["corr"] > np.float32(snr_min)) & np.isfinite(o_r) & np.isfinite(o_a)
    x = locs[use, 0].astype(np.float64)
    y = locs[use, 1].astype(np.float64)
    n = int(use.sum())
    if n:
        cx, cy = 0.5 * (x.min() + x.max()), 0.5 * (y.min() + y.max())
        hx = 0.5 * (x.max() - x.min()) or 1.0
        hy = 0.5 * (y.max() - y.min()) or 1.0
    else:
        cx = cy = 0.0
        hx = hy = 1.0
    u, v = (x - cx) / hx, (y - cy) / hy
    out = {}
    for name, o, npar in (("range", o_r[use].astype(np.float64), npar_range),
                          ("azimuth", o_a[use].astype(np.float64), npar_azimuth)):
        phi = np.stack([np.ones_like(u), u, v], 1)[:, :npar]
        c = np.zeros(3)
        scale = 0.0
        w = np.ones(n)
        for _ in range(robust_iters + 1):
            if scale > 0.0:
                rr = (o - np.stack([np.ones_like(u), u, v], 1) @ c) / (4.685 * scale)
                w = np.where(np.abs(rr) < 1.0, (1.0 - rr * rr) ** 2, 0.0)
            else:
                w = np.ones(n)
            A = (phi * w[:, None]).T @ phi
            b = (phi * w[:, None]).T @ o
            c = np.zeros(3)
            if n:
                c[:npar] = np.linalg.solve(A, b)
            res_ = o - np.stack([np.ones_like(u), u, v], 1) @ c
            scale = float(np.sqrt(np.sum(w * res_ * res_) / np.sum(w))) if np.sum(w) > 0 else 0.0
        stretch, a_stretch = c[1] / hx, c[2] / hy
        shift = c[0] - stretch * cx - a_stretch * cy
        ishift = int(shift)            # truncation toward zero
        out[name] = dict(shift=shift, stretch=stretch, a_stretch=a_stretch, sub_int=shift - ishift, rms=scale,
                         weight=float(np.sum(w)), ishift=ishift, npts=n)
    return out
