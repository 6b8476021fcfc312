"""Seeded random geometries against the oracle: search sizes, anisotropy,
range interpolation and subpixel factors, PRM offsets and azimuth stretch,
image sizes that put windows partly outside the images, and strip lengths
that split the location list unevenly.  Integer and subpixel peaks must match
the oracle's FP32 restatement except where the FP64 oracle calls the subpixel
peak a near-tie; correlation within 1e-4 relative."""
import numpy as np
import pytest

import xcorr_gb300 as xg
import xcorr_oracle as xo
from xcorr_gb300 import synth

pytestmark = pytest.mark.gpu


def _case(seed):
    rng = np.random.default_rng(seed)
    xs = int(rng.choice([32, 64, 128]))
    ys = int(rng.choice([32, 64, 128]))
    ri = int(rng.choice([1, 2, 4]))
    ifc = int(rng.choice([8, 16, 32]))
    nx = int(rng.integers(6 * xs + 64, 6 * xs + 900))
    ny = int(rng.integers(6 * ys + 64, 6 * ys + 900))
    spec = synth.PairSpec(nx=nx, ny=ny, dx=float(rng.uniform(-6, 6)), dy=float(rng.uniform(-6, 6)),
                          noise_frac=float(rng.uniform(0.02, 0.5)), seed=1000 + seed)
    xoff, yoff = int(rng.integers(-9, 10)), int(rng.integers(-9, 10))
    ast = float(rng.choice([0.0, 1e-3, -2e-3]))
    nxl, nyl = int(rng.integers(1, 7)), int(rng.integers(1, 5))
    return xs, ys, ri, ifc, spec, xoff, yoff, ast, nxl, nyl


@pytest.mark.parametrize("seed", range(12))
def test_random_geometry_against_oracle(seed):
    xs, ys, ri, ifc, spec, xoff, yoff, ast, nxl, nyl = _case(seed)
    m, s = synth.make_pair(spec)
    locs = xg.grid(spec.nx, spec.ny, nxl, nyl, xs, ys)
    with xg.Context(xg.params(xs, ys, ri, 1, ifc)) as ctx:
        r = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=nxl)
    o = xo.run(xo.params(xs, ys, ri, 1, ifc), m, s, locs, xoff, yoff, ast, precision=xo.F32, strip_len=nxl)
    np.testing.assert_array_equal(r["flags"], o["flags"])
    ipjp = (r["ip"] == o["ip"]) & (r["jp"] == o["jp"])
    assert ipjp.all(), np.where(~ipjp)[0]
    bad = np.where((r["fip"] != o["fip"]) | (r["fjp"] != o["fjp"]))[0]
    p = xo.params(xs, ys, ri, 1, ifc)
    for i in bad:
        assert xo.near_tie(p, m, s, locs[i, 0], locs[i, 1], (r["fip"][i], r["fjp"][i]), (o["fip"][i], o["fjp"][i]),
                           xoff, yoff, ast), (seed, i)
    ok = o["corr"] != 0
    rel = np.abs(r["corr"][ok].astype(np.float64) - o["corr"][ok]) / np.abs(o["corr"][ok])
    assert rel.size == 0 or rel.max() < 1e-4
