"""The row stage on shared image row segments (the default) against the
per-window row stage of the reference's structure, on the GPU.

Both compute every amplitude with the same instructions, so the patch means,
the (int) copies and the time-domain correlation at equal peaks are the same
bits; the row spectra are transformed with a different pairing (two rows of
one image per complex FFT instead of a window's master and slave row), so
the surfaces differ by FP32 rounding and a peak may move only where the FP64
oracle calls the two candidates a tie."""
import numpy as np
import pytest

import golden_util as gu
import xcorr_gb300 as xg
import xcorr_oracle as xo
from xcorr_gb300 import synth

pytestmark = pytest.mark.gpu


def _both(p, m, s, locs, xoff=0, yoff=0, ast=0.0, strip_len=0):
    with xg.Context(p) as ctx:
        shared = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=strip_len)
        ctx.set_row_sharing(False)
        alone = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=strip_len)
    return shared, alone


def _check(shared, alone, p, m, s, locs, xoff=0, yoff=0, ast=0.0):
    np.testing.assert_array_equal(shared["mean1"], alone["mean1"])
    np.testing.assert_array_equal(shared["mean2"], alone["mean2"])
    same = (shared["ip"] == alone["ip"]) & (shared["jp"] == alone["jp"])
    for i in np.where(~same)[0]:      # only FP64-confirmed ties may differ
        o = xo.run(xo.params(p.xsearch, p.ysearch, p.ri, p.interp_flag, p.interp_factor), m, s, locs[i:i + 1],
                   xoff, yoff, ast, precision=xo.F64)
        assert (o["ip"][0], o["jp"][0]) in {(shared["ip"][i], shared["jp"][i]), (alone["ip"][i], alone["jp"][i])}
    assert (~same).sum() <= max(1, len(locs) // 500)
    np.testing.assert_array_equal(shared["gamma"][same], alone["gamma"][same])
    np.testing.assert_array_equal(shared["flags"], alone["flags"])
    fsame = same & (shared["fip"] == alone["fip"]) & (shared["fjp"] == alone["fjp"])
    assert (same & ~fsame).sum() <= max(1, len(locs) // 200)
    rel = np.abs(shared["cmax"][same] / alone["cmax"][same] - 1)
    assert rel.max() < 1e-5


def test_headline_grid_shares_rows_and_matches():
    g = gu.load("cfg1")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("cfg1", g)
    p = xg.params(64, 64)
    shared, alone = _both(p, m, s, locs, strip_len=d["nxl"])
    _check(shared, alone, p, m, s, locs)
    # and the reference's own integer peaks
    np.testing.assert_array_equal(shared["ip"], g["col"]("ip").astype(np.int32))
    np.testing.assert_array_equal(shared["jp"], g["col"]("jp").astype(np.int32))


@pytest.mark.parametrize("xs,ys,ri,xoff,yoff,ast", [(32, 32, 2, 5, -7, 2e-3), (16, 64, 1, 0, 3, 0.0),
                                                    (128, 32, 4, -2, 0, -1e-3), (64, 128, 2, 0, 0, 0.0)])
def test_shapes_offsets_stretch(xs, ys, ri, xoff, yoff, ast):
    nx, ny = max(1024, 10 * xs), max(1536, 14 * ys)
    m, s = synth.make_pair(synth.PairSpec(nx=nx, ny=ny, dx=1.4, dy=-2.2, noise_frac=0.1, seed=7 * xs + ys))
    locs = xg.grid(nx, ny, 5, 9, xs, ys)
    extra = np.array([[10, ny // 2], [nx - 5, ny // 3], [nx // 2, 5]], np.int32)     # partly outside
    locs = np.concatenate([locs, locs[:3], extra]).astype(np.int32)                  # duplicates too
    p = xg.params(xs, ys, ri)
    shared, alone = _both(p, m, s, locs, xoff, yoff, ast, strip_len=5)
    _check(shared, alone, p, m, s, locs, xoff, yoff, ast)
    assert (shared["flags"][-3:] & xg.FLAG_OOB).all()


def test_device_entry_batches_and_streams():
    """Several batches on the two scratch slots, through the device entry."""
    torch = pytest.importorskip("torch")
    m, s = synth.make_pair(synth.PairSpec(nx=2048, ny=3072, dx=-0.7, dy=1.9, noise_frac=0.1, seed=31))
    locs = xg.grid(2048, 3072, 12, 30, 64, 64)
    dev = torch.device("cuda", 0)
    dm, ds, dl = torch.from_numpy(m).to(dev), torch.from_numpy(s).to(dev), torch.from_numpy(locs).to(dev)
    n = len(locs)
    outs = []
    for sharing in (True, False):
        with xg.Context(xg.params(64, 64), max_batch=96) as ctx:
            ctx.set_row_sharing(sharing)
            out = torch.zeros((n, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
            ctx.correlate_device(dm.data_ptr(), 2048, 3072, ds.data_ptr(), 2048, 3072, dl.data_ptr(), n,
                                 out.data_ptr(), torch.cuda.current_stream(dev).cuda_stream, strip_len=12)
            torch.cuda.synchronize()
            assert ctx.stats().batches == 4
            outs.append(np.frombuffer(out.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE))
    _check(outs[0], outs[1], xg.params(64, 64), m, s, locs)


@pytest.mark.parametrize("xs,ys", [(64, 64), (16, 16), (32, 128), (128, 32), (256, 64), (16, 256)])
def test_column_stage_forms_give_the_same_bits(xs, ys):
    """The persistent column stage (each CTA a range of (window, column
    group) tiles, the next tile's rows staged during the current one) and
    one CTA per tile do the same arithmetic: every result field identical,
    also where a CTA's range starts or ends inside a window."""
    nx, ny = max(1024, 10 * xs), max(1536, 14 * ys)
    m, s = synth.make_pair(synth.PairSpec(nx=nx, ny=ny, dx=0.8, dy=-1.3, noise_frac=0.1, seed=3 * xs + ys))
    locs = xg.grid(nx, ny, 7, 11, xs, ys)
    p = xg.params(xs, ys)
    with xg.Context(p) as ctx:
        persistent = ctx.correlate(m, s, locs, 3, -4, 1e-3, strip_len=7)
        ctx.set_launch_shapes(1)
        per_tile = ctx.correlate(m, s, locs, 3, -4, 1e-3, strip_len=7)
        ctx.set_launch_shapes(0, 2)                  # and the peak stage at 512 threads per window
        wide_peak = ctx.correlate(m, s, locs, 3, -4, 1e-3, strip_len=7)
        ctx.set_launch_shapes(2)                     # the other persistent form (slave spectrum in registers or not)
        kept = ctx.correlate(m, s, locs, 3, -4, 1e-3, strip_len=7)
    assert persistent.tobytes() == per_tile.tobytes()
    assert wide_peak.tobytes() == per_tile.tobytes()
    assert kept.tobytes() == per_tile.tobytes()
