"""Full-frame configuration at full size: 10240 x 30720 pair with a
spatially varying shift, 40000 locations of 256x256 windows (512x512 FFTs).

Against the reference's own run on the same inputs (tests/golden/ref_cfg2.npz,
made by make_ref_cfg2.py on the GB300): integer and subpixel peaks identical,
corr within 1e-4; against the FP64 oracle on a sample of windows; and the
recovered offsets against the generator's shift field."""
import os

import numpy as np
import pytest

import xcorr_gb300 as xg
import xcorr_oracle as xo
from xcorr_gb300 import synth

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_cfg2.npz")


@pytest.fixture(scope="module")
def cfg2():
    if not os.path.exists(GOLD):
        pytest.skip("no full-frame reference record")
    import make_ref_cfg2 as mk
    g = np.load(GOLD)
    m, s, truth = mk.make_inputs()
    if synth.sha256(m) != str(g["sha_master"]) or synth.sha256(s) != str(g["sha_slave"]):
        pytest.skip("regenerated full-frame inputs differ from the recorded ones (different torch/cuFFT build)")
    locs = xg.grid(mk.NX, mk.NY, 100, 400, 128, 128)
    with xg.Context(xg.params(128, 128)) as ctx:
        r = ctx.correlate(m, s, locs, strip_len=100)
    return g, m, s, truth, locs, r


def test_full_frame_matches_reference(cfg2):
    g, m, s, truth, locs, r = cfg2
    assert (g["x"] == locs[:, 0]).all() and (g["y"] == locs[:, 1]).all()
    np.testing.assert_array_equal(r["ip"], g["ip"].astype(np.int32))
    np.testing.assert_array_equal(r["jp"], g["jp"].astype(np.int32))
    # subpixel peaks: identical, except near-ties (neighbouring cells whose
    # FP64 values agree within 1e-5 of the peak), at most 1 in 10^4 windows
    bad = np.nonzero((r["fip"] != g["fip"]) | (r["fjp"] != g["fjp"]))[0]
    assert len(bad) <= len(locs) // 10000, f"{len(bad)} of {len(locs)} subpixel peaks differ"
    for i in bad:
        assert xo.near_tie(xo.params(128, 128), m, s, locs[i, 0], locs[i, 1], (int(r["fip"][i]), int(r["fjp"][i])),
                           (int(g["fip"][i]), int(g["fjp"][i]))), f"window {i} differs and is not a tie"
    rel = np.abs(r["corr"] - g["corr"]) / np.maximum(np.abs(g["corr"]), 1e-30)
    assert rel.max() < 1e-4


def test_full_frame_against_truth_and_fp64_oracle(cfg2):
    g, m, s, truth, locs, r = cfg2
    xo_, yo_ = xg.output_offsets(r, 2, 0, 0, locs[:, 1], 0.0)
    tx, ty = truth(locs[:, 0], locs[:, 1])
    ex, ey = xo_ - tx, yo_ - ty
    # amplitude correlation of speckle: subpixel bias of the 1/16-px FFT interpolation
    assert np.sqrt(np.mean(ex ** 2)) < 0.1 and np.sqrt(np.mean(ey ** 2)) < 0.15
    idx = np.linspace(0, len(locs) - 1, 24).astype(int)
    o = xo.run(xo.params(128, 128), m, s, locs[idx], precision=xo.F64, strip_len=0)
    for k in ("ip", "jp", "fip", "fjp"):
        np.testing.assert_array_equal(r[k][idx], o[k], err_msg=k)
    assert np.max(np.abs(r["gamma"][idx] - o["gamma"]) / o["gamma"]) < 1e-4
