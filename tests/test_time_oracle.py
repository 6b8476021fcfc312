"""The -time / -time4 restatement in the oracle (do_time_corr,
do_time_int_xcorr.cu:146-189).  The reference's GPU program runs these modes
without data, so its own functions were driven directly
(oracle/_ref/ref_time_probe, tests/golden/make_ref_time.py) on the integer
patches of golden windows: the oracle must reproduce their float64 surfaces
bit for bit and the peak and correlation they set.  Beyond that it is pinned
to the frequency path: the full-search surface at the frequency path's
integer peak is the same calc_time_corr formula the frequency path evaluates
there, so where both modes pick the same lag their correlation is identical,
and on a clean pair both pick the true shift."""
import gzip
import hashlib
import json
import os

import numpy as np
import pytest

import golden_util as gu
import xcorr_oracle as xo
from xcorr_gb300 import synth
from xcorr_gb300.synth import PairSpec


def load_time_records():
    with gzip.open(os.path.join(gu.GOLDEN_DIR, "ref_time.json.gz"), "rt") as f:
        return json.load(f)["records"]


def window_ints(case, w):
    """The integer patches of one golden window as the fixture generator made them."""
    g = gu.load(case)
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs(case, g)
    x, y = (int(v) for v in locs[w])
    p = xo.params(d["xsearch"], d["ysearch"], d["ri"])
    pm, ps = gu.cut_patches(m, s, x, y, p.npx, p.npy, xoff, yoff, ast)
    return d, locs[w], xo.prepare_patch(p, pm, False, xo.F32)[2], xo.prepare_patch(p, ps, True, xo.F32)[2]


@pytest.mark.parametrize("rec", load_time_records(), ids=lambda r: f"{r['case']}-w{r['window']}-mode{r['mode']}")
def test_time_surface_matches_reference_functions(rec):
    d, loc, i1, i2 = window_ints(rec["case"], rec["window"])
    assert hashlib.sha256(i1.tobytes()).hexdigest() == rec["i1_sha256"]
    assert hashlib.sha256(i2.tobytes()).hexdigest() == rec["i2_sha256"]
    p = xo.params(d["xsearch"], d["ysearch"], d["ri"], corr_mode=rec["mode"])
    corr, r = xo.time_surface(p, i1, i2)
    np.testing.assert_array_equal(corr.ravel()[rec["sample_index"]], np.array(rec["sample_value"]))
    assert hashlib.sha256(corr.tobytes()).hexdigest() == rec["surface_sha256"], "surface differs in some bit"
    assert float(np.abs(corr).max()) == rec["surface_max"]
    assert (float(r["xoff"]), float(r["yoff"]), float(r["corr"])) == (rec["xoff"], rec["yoff"], rec["corr"])


@pytest.fixture(scope="module")
def xs32():
    g = gu.load("xs32")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("xs32", g)
    return m, s, locs[:48], xoff, yoff, ast


def test_time_mode_agrees_with_frequency_path(xs32):
    m, s, locs, xoff, yoff, ast = xs32
    f = xo.run(xo.params(32, 32), m, s, locs, xoff, yoff, ast, precision=xo.F32, strip_len=8)
    t = xo.run(xo.params(32, 32, corr_mode=0), m, s, locs, xoff, yoff, ast, precision=xo.F32, strip_len=8)
    same = (f["ip"] == t["ip"]) & (f["jp"] == t["jp"])
    assert same.mean() > 0.9
    # same lag, same formula, same ints: the correlation is identical
    np.testing.assert_array_equal(t["corr"][same], f["corr"][same])
    # the time surface's maximum is the reported peak value
    np.testing.assert_array_equal(t["corr"], t["cmax"].astype(np.float32))


def test_time4_clean_pair_finds_the_shift():
    m, s = synth.make_pair(PairSpec(nx=768, ny=768, dx=2.0, dy=-3.0, noise_frac=0.002, seed=21))
    locs = np.array([[384, 384], [320, 400], [448, 360]], np.int32)
    t4 = xo.run(xo.params(32, 32, corr_mode=1), m, s, locs, precision=xo.F64)
    t0 = xo.run(xo.params(32, 32, corr_mode=0), m, s, locs, precision=xo.F64)
    np.testing.assert_array_equal(t4["xoff"], 4.0)          # 2 px at range interpolation 2
    np.testing.assert_array_equal(t4["yoff"], -3.0)
    np.testing.assert_array_equal(t0["xoff"], 4.0)
    assert (t4["corr"] > 50).all() and (t0["corr"] > 90).all()


def test_time4_noisy_pair_gives_zero_surface():
    # the 4th-power estimate sqrt(2 r - 1) is defined only for r > 0.5; a noisy
    # pair stays below and every lag scores 0, so the scan keeps the first lag
    m, s = synth.make_pair(PairSpec(nx=512, ny=512, dx=2.3, dy=-1.6, noise_frac=0.2, seed=3))
    r = xo.run(xo.params(32, 32, corr_mode=1), m, s, np.array([[256, 256]], np.int32), precision=xo.F64)
    assert r["corr"][0] == 0.0 and r["xoff"][0] == 32.0 and r["yoff"][0] == 32.0
