"""The surrogate form on the headline configuration's inputs (the cfg1
golden case: 2048 x 4096 pair, shift (3.37, -5.81) px, 10% noise, 1000
windows of 128 x 128): range interpolation 1 (no 2x range oversampling) with
the subpixel refiner trained on ri = 1 surfaces standing in for the FFT
zero-pad interpolation, which still answers for the windows the refiner
declines.

* The plain form's offsets equal the FP64 oracle's on a 100-window sample, so
  the benchmark's "RMS against the plain form" is RMS against the FP64 oracle.
* Declined windows are bit-identical to the plain ri = 1 path; refined ones
  carry XCG_FLAG_REFINED.  The refiner is taken where its sigma is below
  0.15 px and it agrees with a 3-point parabola within 0.4 px (a parabola
  through 1-px samples is biased by up to about 0.3 px).
* The claimed reading of the benchmark spec's accuracy bar: per axis, the
  surrogate's RMS error against the synthetic truth is at most the FP64
  oracle's RMS error plus 0.02 px.
* What the refiner gains: it beats the FFT interpolation of the same ri = 1
  surfaces against the truth."""
import os

import numpy as np
import pytest

import golden_util as gu
import xcorr_gb300 as xg
import xcorr_oracle as xo
from xcorr_gb300 import refiner_train as rt

pytestmark = pytest.mark.gpu

TRUTH = (3.37, -5.81)


def _rms(e):
    return float(np.sqrt(np.mean(np.square(e))))


@pytest.fixture(scope="module")
def cfg1():
    g = gu.load("cfg1")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("cfg1", g)
    return m, s, locs, d


def test_plain_form_equals_fp64_oracle_on_sample(cfg1):
    m, s, locs, d = cfg1
    sub = np.ascontiguousarray(locs[::10])
    with xg.Context(xg.params(64, 64)) as ctx:
        r = ctx.correlate(m, s, sub, strip_len=0)
    o = xo.run(xo.params(64, 64), m, s, sub, precision=xo.F64, strip_len=0)
    xr, yr = xg.output_offsets(r, 2, 0, 0, sub[:, 1], 0.0)
    xf, yf = xg.output_offsets(o, 2, 0, 0, sub[:, 1], 0.0)
    np.testing.assert_array_equal(xr, xf)
    np.testing.assert_array_equal(yr, yf)


@pytest.mark.skipif(not os.path.exists(rt.weights_path(1)), reason="no trained ri = 1 refiner parameters")
def test_surrogate_form_accuracy_and_fallback(cfg1):
    torch = pytest.importorskip("torch")
    m, s, locs, d = cfg1
    dev = torch.device("cuda", 0)
    dm, ds = torch.from_numpy(m).to(dev), torch.from_numpy(s).to(dev)
    dl = torch.from_numpy(locs).to(dev)
    n = len(locs)
    sp = torch.cuda.current_stream(dev).cuda_stream
    with xg.Context(xg.params(64, 64)) as ctx:
        plain2 = ctx.correlate(m, s, locs, strip_len=20)
    with xg.Context(xg.params(64, 64, 1, 1, 16)) as ctx1:
        plain1 = ctx1.correlate(m, s, locs, strip_len=20)
        ref = xg.Refiner(0, max_batch=64)
        ref.set_params(rt.load_weights(rt.weights_path(1)))
        out = torch.zeros((n, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
        ctx1.correlate_device_refined(ref, dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1],
                                      s.shape[0], dl.data_ptr(), n, out.data_ptr(), sp, strip_len=20,
                                      max_sigma=0.15, max_disagree=0.4)
        torch.cuda.synchronize()
        ref.close()
    sur = np.frombuffer(out.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)
    refined = (sur["flags"] & xg.FLAG_REFINED) != 0
    assert refined.mean() > 0.9
    # declined windows: the plain ri = 1 answer, bit for bit
    for k in ("ip", "jp", "fip", "fjp", "xfrac", "yfrac", "xoff", "yoff", "corr"):
        np.testing.assert_array_equal(sur[k][~refined], plain1[k][~refined], err_msg=k)
    np.testing.assert_array_equal(sur["ip"], plain1["ip"])
    x2, y2 = xg.output_offsets(plain2, 2, 0, 0, locs[:, 1], 0.0)
    x1, y1 = xg.output_offsets(plain1, 1, 0, 0, locs[:, 1], 0.0)
    xs, ys = xg.output_offsets(sur, 1, 0, 0, locs[:, 1], 0.0)
    e_oracle = (_rms(x2 - TRUTH[0]), _rms(y2 - TRUTH[1]))
    e_sur = (_rms(xs - TRUTH[0]), _rms(ys - TRUTH[1]))
    e_fft1 = (_rms(x1 - TRUTH[0]), _rms(y1 - TRUTH[1]))
    assert e_sur[0] <= e_oracle[0] + 0.02 and e_sur[1] <= e_oracle[1] + 0.02, (e_sur, e_oracle)
    assert e_sur[0] < e_fft1[0] and e_sur[1] < e_fft1[1], (e_sur, e_fft1)
