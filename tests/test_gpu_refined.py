"""The refined path (xcg_correlate_device_refined) with the committed trained
refiner: on held-out synthetic tiles it must leave integer peaks and the
time-domain correlation untouched, give windows it does not accept exactly
the plain subpixel result, and -- what the network buys -- a lower error
against the true shift than the plain FFT interpolation."""
import os

import numpy as np
import pytest

import xcorr_gb300 as xg

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gmtsar-gpu_gb300", "refiner",
                       "subpix_refiner.f32")


@pytest.fixture(scope="module")
def run():
    torch = pytest.importorskip("torch")
    if not os.path.exists(WEIGHTS):
        pytest.skip("no trained refiner weights")
    from xcorr_gb300 import refiner_train as rt
    dev = torch.device("cuda", 0)
    m, s, locs, shift, snr = rt.make_tiles(32, 32, 987654321, dev)       # a seed the training never used
    n = len(locs)
    ny, nx = m.shape[0], m.shape[1]
    dl = torch.from_numpy(locs).to(dev)
    plain = torch.zeros((n, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    refd = torch.zeros_like(plain)
    ref = xg.Refiner(0, max_batch=64)
    ref.set_params(rt.load_weights(WEIGHTS))
    st = torch.cuda.current_stream(dev).cuda_stream
    with xg.Context(xg.params(64, 64)) as ctx:
        ctx.correlate_device(m.data_ptr(), nx, ny, s.data_ptr(), nx, ny, dl.data_ptr(), n, plain.data_ptr(), st)
        ctx.correlate_device_refined(ref, m.data_ptr(), nx, ny, s.data_ptr(), nx, ny, dl.data_ptr(), n,
                                     refd.data_ptr(), st, max_sigma=0.15, max_disagree=0.25)
    torch.cuda.synchronize()
    h = lambda t: np.frombuffer(t.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)
    return h(plain), h(refd), locs, shift, snr


def test_refined_keeps_the_plain_answers(run):
    p, r, locs, shift, snr = run
    for k in ("ip", "jp", "xoff", "yoff", "corr", "gamma", "cmax"):
        np.testing.assert_array_equal(p[k], r[k], err_msg=k)
    used = (r["flags"] & xg.FLAG_REFINED) != 0
    assert 0.5 < used.mean() <= 1.0
    for k in ("xfrac", "yfrac", "fip", "fjp"):
        np.testing.assert_array_equal(p[k][~used], r[k][~used], err_msg=k)


def test_refined_beats_the_fft_interpolation_against_truth(run):
    p, r, locs, shift, snr = run
    xp, yp = xg.output_offsets(p, 2, 0, 0, locs[:, 1], 0.0)
    xr, yr = xg.output_offsets(r, 2, 0, 0, locs[:, 1], 0.0)
    good = (np.abs(xp - shift[:, 0]) < 1) & (np.abs(yp - shift[:, 1]) < 1)
    rms = lambda e: float(np.sqrt(np.mean(e[good] ** 2)))
    ex_p, ex_r = rms(xp - shift[:, 0]), rms(xr - shift[:, 0])
    ey_p, ey_r = rms(yp - shift[:, 1]), rms(yr - shift[:, 1])
    assert ex_r < 0.6 * ex_p, (ex_r, ex_p)
    assert ey_r < ey_p, (ey_r, ey_p)


def test_refined_path_any_batch_split():
    """The refined path runs its batches through the plain path's scheduler:
    one batch, two slots or the four half-slot lanes give the same bits."""
    torch = pytest.importorskip("torch")
    if not os.path.exists(WEIGHTS):
        pytest.skip("no trained refiner weights")
    from xcorr_gb300 import refiner_train as rt
    dev = torch.device("cuda", 0)
    m, s, locs, shift, snr = rt.make_tiles(32, 32, 55555, dev)
    n = len(locs)
    ny, nx = m.shape[0], m.shape[1]
    dl = torch.from_numpy(locs).to(dev)
    ref = xg.Refiner(0, max_batch=64)
    ref.set_params(rt.load_weights(WEIGHTS))
    st = torch.cuda.current_stream(dev).cuda_stream
    outs = []
    with xg.Context(xg.params(64, 64)) as ctx:
        with pytest.raises(xg.XcgError):
            ctx.set_batches(-1)
        for nb in (1, 2, 3, 4, 8):
            ctx.set_batches(nb)
            out = torch.zeros((n, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
            ctx.correlate_device_refined(ref, m.data_ptr(), nx, ny, s.data_ptr(), nx, ny, dl.data_ptr(), n,
                                         out.data_ptr(), st, max_sigma=0.15, max_disagree=0.25)
            torch.cuda.synchronize()
            assert ctx.stats().batches == nb
            outs.append(out.cpu().numpy().tobytes())
    ref.close()
    assert all(o == outs[0] for o in outs[1:])
