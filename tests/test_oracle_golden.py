"""The oracle against the reference's own outputs (golden vectors made by
running the reference xcorr-gpu on the GB300 machine, tests/golden/make_ref_golden.py).

Bar: integer peaks and fine (subpixel) peaks identical; correlation, surface
maximum and reference mean within 1e-4 relative; patch means within 1e-6."""
import numpy as np
import pytest

import golden_util as gu
import xcorr_oracle as xo
from cases import CASES
from xcorr_gb300 import synth


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = np.isfinite(b) & (b != 0)
    return float(np.max(np.abs(a[ok] - b[ok]) / np.abs(b[ok]))) if ok.any() else 0.0


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("precision", [xo.F32, xo.F64])
def test_oracle_matches_reference(name, precision):
    g = gu.load(name)
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs(name, g)
    # the inputs are regenerated bit for bit
    assert synth.sha256(m) == g["sha256"]["master"]
    assert synth.sha256(s) == g["sha256"]["slave"]
    assert (g["col"]("x") == locs[:, 0]).all() and (g["col"]("y") == locs[:, 1]).all()
    p = xo.params(d["xsearch"], d["ysearch"], d["ri"], d["interp_flag"], d["ifc"])
    r = xo.run(p, m, s, locs, xoff, yoff, ast, precision=precision, strip_len=d["nxl"])
    for k in ("ip", "jp", "fip", "fjp"):
        np.testing.assert_array_equal(r[k], g["col"](k).astype(np.int32), err_msg=k)
    np.testing.assert_array_equal(r["xoff"], g["col"]("xoff").astype(np.float32))
    np.testing.assert_array_equal(r["yoff"], g["col"]("yoff").astype(np.float32))
    np.testing.assert_array_equal(r["xfrac"], g["col"]("xfrac").astype(np.float32))
    np.testing.assert_array_equal(r["yfrac"], g["col"]("yfrac").astype(np.float32))
    assert _rel(r["corr"], g["col"]("corr")) < 1e-4
    assert _rel(r["cmax"], g["col"]("cmax")) < 1e-4
    assert _rel(r["cave"], g["col"]("cave")) < 1e-4
    assert _rel(r["mean1"], g["col"]("mean1")) < 1e-6
    assert _rel(r["mean2"], g["col"]("mean2")) < 1e-6
    # gamma = 0 exactly where the reference printed 0 (zero patches)
    np.testing.assert_array_equal(r["corr"] == 0, g["col"]("corr") == 0)


def test_argmax_tie_rules():
    """Ties and non-positive values follow reduce6b's tournament
    (conv_ampl_demean.cu:434-554) and the host's block scan (:655-673)."""
    x = np.zeros(4096)
    assert xo.argmax_ref(x)[0] == 0                 # all zero: first element
    x[[5, 3]] = 7.0
    # 5 = 0b101 -> bit-reversed 0b10100000000, 3 = 0b011 -> 0b11000000000: 5 wins
    assert xo.argmax_ref(x)[0] == 5
    x = np.zeros(4096); x[1030] = 2.0; x[2048 + 1] = 2.0
    assert xo.argmax_ref(x)[0] == 1030              # earlier block wins a tie
    x = -np.ones(4096)
    assert xo.argmax_ref(x)[0] == 0                 # negatives act as the initial 0
    x = np.full(4096, np.nan)
    assert xo.argmax_ref(x)[0] == 0
