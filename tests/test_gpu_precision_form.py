"""The precision form (split-FP16 tcgen05 DFTs for the correlation's row and
column transforms) on the 128x128-window golden case, against the
reference's own outputs, the FP32 SIMT path and the FP64 oracle.  Split FP16
carries about 22 bits per operand, so the surface differs from the FP32
path's at the 1e-6 level; on this case that changes no peak: integer peaks
equal the reference's and subpixel peaks the FP32 path's, all 1000 of them."""
import numpy as np
import pytest

import golden_util as gu
import xcorr_gb300 as xg
import xcorr_oracle as xo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg1():
    g = gu.load("cfg1")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("cfg1", g)
    p = xg.params(64, 64)
    with xg.Context(p) as ctx:
        r32 = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=d["nxl"])
        ctx.set_dft_form(1)
        rtc = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=d["nxl"])
        ctx.set_dft_form(0)
        r32b = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=d["nxl"])
    return g, m, s, locs, d, r32, rtc, r32b


def test_switching_back_restores_the_fp32_path(cfg1):
    g, m, s, locs, d, r32, rtc, r32b = cfg1
    assert r32.tobytes() == r32b.tobytes()


def test_precision_form_matches_reference(cfg1):
    g, m, s, locs, d, r32, rtc, _ = cfg1
    ip, jp = g["col"]("ip").astype(np.int32), g["col"]("jp").astype(np.int32)
    bad = np.where((rtc["ip"] != ip) | (rtc["jp"] != jp))[0]
    assert len(bad) == 0, bad
    np.testing.assert_array_equal(rtc["fip"], r32["fip"])
    np.testing.assert_array_equal(rtc["fjp"], r32["fjp"])
    xo_t, yo_t = xg.output_offsets(rtc, 2, 0, 0, locs[:, 1], 0.0)
    xo_f, yo_f = xg.output_offsets(r32, 2, 0, 0, locs[:, 1], 0.0)
    assert np.max(np.abs(xo_t - xo_f)) <= 0.0625 and np.mean(np.abs(xo_t - xo_f) <= 0.01) >= 0.99
    rel = np.abs(rtc["corr"].astype(np.float64) - r32["corr"]) / r32["corr"]
    assert np.median(rel) < 1e-5 and rel.max() < 1e-3, (np.median(rel), rel.max())
    assert np.max(np.abs(rtc["cmax"] / r32["cmax"] - 1)) < 1e-4


def test_precision_form_error_against_fp64(cfg1):
    """Both forms' offsets against the FP64 oracle, reported side by side."""
    g, m, s, locs, d, r32, rtc, _ = cfg1
    sub = np.arange(0, len(locs), 10)
    o = xo.run(xo.params(64, 64), m, s, locs[sub], precision=xo.F64, strip_len=0)
    xo_o, yo_o = xg.output_offsets(o, 2, 0, 0, locs[sub, 1], 0.0)
    out = {}
    for name, r in (("fp32", r32), ("split_fp16_tc", rtc)):
        x, y = xg.output_offsets(r[sub], 2, 0, 0, locs[sub, 1], 0.0)
        out[name] = (float(np.sqrt(np.mean((x - xo_o) ** 2))), float(np.sqrt(np.mean((y - yo_o) ** 2))))
    print("rms offset error vs FP64 oracle [range, azimuth] px:", out)
    assert out["split_fp16_tc"][0] <= out["fp32"][0] + 0.01
    assert out["split_fp16_tc"][1] <= out["fp32"][1] + 0.01


def test_refined_path_in_precision_form(cfg1):
    """The refined path runs the tensor-core stages too and agrees with its
    FP32 form (the refiner sees the same neighbourhoods to ~1e-6)."""
    import os
    torch = pytest.importorskip("torch")
    from xcorr_gb300 import refiner_train as rt
    wpath = os.path.join(os.path.dirname(xg.__file__), "..", "..", "refiner", "subpix_refiner.f32")
    if not os.path.exists(wpath):
        pytest.skip("no trained refiner weights")
    g, m, s, locs, d, r32, rtc, _ = cfg1
    dev = torch.device("cuda")
    dm, ds = torch.from_numpy(m).to(dev), torch.from_numpy(s).to(dev)
    dl = torch.from_numpy(locs).to(dev)
    out = []
    ref = xg.Refiner(0, max_batch=64)
    ref.set_params(rt.load_weights(wpath))
    with xg.Context(xg.params(64, 64)) as ctx:
        for form in (0, 1):
            ctx.set_dft_form(form)
            dr = torch.zeros((len(locs), xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
            ctx.correlate_device_refined(ref, dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1],
                                         s.shape[0], dl.data_ptr(), len(locs), dr.data_ptr(), strip_len=d["nxl"],
                                         max_sigma=0.15)
            torch.cuda.synchronize()
            out.append(np.frombuffer(dr.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE))
    ref.close()
    a, b = out
    np.testing.assert_array_equal(a["ip"], b["ip"])
    np.testing.assert_array_equal(a["jp"], b["jp"])
    assert np.mean(a["flags"] == b["flags"]) > 0.99
    # the refiner's inference quantises its inputs to BF16, so a feature that
    # moves by 1e-6 can move its output by ~1e-3 px: well inside 0.01 px
    both = ((a["flags"] & xg.FLAG_REFINED) != 0) & ((b["flags"] & xg.FLAG_REFINED) != 0)
    assert np.max(np.abs(a["xfrac"][both] - b["xfrac"][both])) < 5e-3
    assert np.max(np.abs(a["yfrac"][both] - b["yfrac"][both])) < 5e-3


@pytest.mark.parametrize("case", ["xs32", "norange_i8", "prmshift"])
def test_precision_form_64_windows(case):
    """64x64 windows (128-point transforms): the same agreement with the FP32
    path and the reference's integer peaks."""
    g = gu.load(case)
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs(case, g)
    p = xg.params(d["xsearch"], d["ysearch"], d["ri"], d["interp_flag"], d["ifc"], fmt=1 if d["real"] else 0)
    with xg.Context(p) as ctx:
        r32 = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=d["nxl"])
        ctx.set_dft_form(1)
        rtc = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=d["nxl"])
    np.testing.assert_array_equal(rtc["ip"], g["col"]("ip").astype(np.int32))
    np.testing.assert_array_equal(rtc["jp"], g["col"]("jp").astype(np.int32))
    same = (rtc["fip"] == r32["fip"]) & (rtc["fjp"] == r32["fjp"])
    assert same.mean() >= 0.97, same.mean()
    rel = np.abs(rtc["cmax"] / r32["cmax"] - 1)
    assert rel.max() < 1e-4


def test_precision_form_rejects_other_shapes():
    with xg.Context(xg.params(32, 64)) as ctx:
        with pytest.raises(xg.XcgError):
            ctx.set_dft_form(1)


def test_stage_timeout_is_reported_then_cleared(cfg1):
    """A tensor-core wait that runs out (injected on the host: the flag the
    stages raise is set at the start of the call) fails the host entry, marks
    every window of the device entry, and does not outlive its call."""
    torch = pytest.importorskip("torch")
    g, m, s, locs, d, r32, rtc, _ = cfg1
    sub = locs[:40]
    with xg.Context(xg.params(64, 64)) as ctx:
        ctx.set_dft_form(1)
        ctx.inject_stage_timeout()
        with pytest.raises(xg.XcgError, match="wait ran out"):
            ctx.correlate(m, s, sub, strip_len=d["nxl"])
        r = ctx.correlate(m, s, sub, strip_len=d["nxl"])          # the next call is clean
        assert not (r["flags"] & xg.FLAG_STAGE_TIMEOUT).any()
        np.testing.assert_array_equal(r["ip"], rtc["ip"][:40])
        dev = torch.device("cuda", 0)
        dm, ds = torch.from_numpy(m).to(dev), torch.from_numpy(s).to(dev)
        dl = torch.from_numpy(np.ascontiguousarray(sub)).to(dev)
        out = torch.zeros((len(sub), xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
        sp = torch.cuda.current_stream(dev).cuda_stream
        for inject in (True, False):
            if inject:
                ctx.inject_stage_timeout()
            ctx.correlate_device(dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1], s.shape[0],
                                 dl.data_ptr(), len(sub), out.data_ptr(), sp, strip_len=d["nxl"])
            torch.cuda.synchronize()
            fl = np.frombuffer(out.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)["flags"]
            assert ((fl & xg.FLAG_STAGE_TIMEOUT) != 0).all() == inject and ((fl & xg.FLAG_STAGE_TIMEOUT) != 0).any() == inject
