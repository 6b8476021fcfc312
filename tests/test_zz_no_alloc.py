"""The allocation-free entry point, xcg_correlate_device_noalloc.

It serves callers that must not allocate device memory (code inside another
framework's memory budget, or on a latency-critical stream where cudaMalloc
would synchronise the device); all its scratch is one fixed 32 MiB array in
the library.  Here it must give the same results as the context entry point
(xcg_correlate_device) on two calls in a row -- the second call finds the
first call's leftovers in the shared array -- and refuse a call that does not
fit with a clear error.  The test allocates inputs and outputs itself (torch),
as such a caller would.  This file is named to be collected last."""
import time

import numpy as np
import pytest

import golden_util as gu
import xcorr_gb300 as xg

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = np.isfinite(b) & (b != 0)
    return float(np.max(np.abs(a[ok] - b[ok]) / np.abs(b[ok]))) if ok.any() else 0.0


def _to_host(t):
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)


def test_noalloc_matches_context_entry_on_two_calls():
    torch = pytest.importorskip("torch")
    g = gu.load("xs32")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("xs32", g)
    p = xg.params(d["xsearch"], d["ysearch"], d["ri"], d["interp_flag"], d["ifc"])
    dev = torch.device("cuda", 0)
    dm, ds = torch.from_numpy(m).to(dev), torch.from_numpy(s).to(dev)
    dl = torch.from_numpy(locs).to(dev)
    n = len(locs)
    sp = torch.cuda.current_stream(dev).cuda_stream
    want = torch.zeros((n, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    with xg.Context(p) as ctx:
        ctx.correlate_device(dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1], s.shape[0],
                             dl.data_ptr(), n, want.data_ptr(), sp, xoff, yoff, ast, strip_len=d["nxl"])
    torch.cuda.synchronize()
    want = _to_host(want)
    for call, fill in enumerate((0xA5, 0x3C)):
        got = torch.full((n, xg.RESULT_DTYPE.itemsize), fill, dtype=torch.uint8, device=dev)
        xg.correlate_device_noalloc(p, dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1], s.shape[0],
                                    dl.data_ptr(), n, got.data_ptr(), sp, xoff, yoff, ast, strip_len=d["nxl"])
        torch.cuda.synchronize()
        got = _to_host(got)
        for k in ("ip", "jp", "fip", "fjp", "flags"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"call {call}: {k}")
        for k in ("xoff", "yoff", "xfrac", "yfrac"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"call {call}: {k}")
        for k in ("corr", "gamma", "cmax", "cave", "cave_true", "mean1", "mean2"):
            assert _rel(got[k], want[k]) < 1e-4, (call, k)
        # and the reference's own numbers
        np.testing.assert_array_equal(got["ip"], g["col"]("ip").astype(np.int32))
        np.testing.assert_array_equal(got["fjp"], g["col"]("fjp").astype(np.int32))


def test_noalloc_refuses_more_than_its_fixed_scratch():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    p = xg.params(64, 64)                      # about 1 MiB of scratch per window
    img = torch.zeros((4096, 2048, 2), dtype=torch.int16, device=dev)
    locs = torch.from_numpy(xg.grid(2048, 4096, 8, 8)).to(dev)   # 64 windows > 32 MiB
    out = torch.zeros((64, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    with pytest.raises(xg.XcgError, match="size exceeds a fixed limit.*at most"):
        xg.correlate_device_noalloc(p, img.data_ptr(), 2048, 4096, img.data_ptr(), 2048, 4096,
                                    locs.data_ptr(), 64, out.data_ptr(), 0)


def test_noalloc_call_does_not_wait_for_the_stream():
    """The entry copies nothing from host memory (its tables are computed on
    the device), so a call queued behind long-running work returns at once and
    still gives the context entry's results once the stream drains."""
    torch = pytest.importorskip("torch")
    g = gu.load("xs32")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("xs32", g)
    p = xg.params(d["xsearch"], d["ysearch"], d["ri"], d["interp_flag"], d["ifc"])
    dev = torch.device("cuda", 0)
    dm, ds = torch.from_numpy(m).to(dev), torch.from_numpy(s).to(dev)
    dl = torch.from_numpy(locs).to(dev)
    n = len(locs)
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream
    got = torch.zeros((n, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    args = (p, dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1], s.shape[0], dl.data_ptr(), n,
            got.data_ptr(), sp, xoff, yoff, ast)
    xg.correlate_device_noalloc(*args, strip_len=d["nxl"])       # set-up call
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        got.fill_(0xA5)                          # so the results read below are the second call's
        torch.cuda._sleep(400_000_000)           # about 0.2 s of queued GPU work at 2 GHz
    t0 = time.perf_counter()
    xg.correlate_device_noalloc(*args, strip_len=d["nxl"])
    host_s = time.perf_counter() - t0
    stream.synchronize()
    total_s = time.perf_counter() - t0
    assert total_s > 0.05, "the queued work did not run"
    assert host_s < 0.5 * total_s, f"the call waited for the stream: {host_s:.3f} s of {total_s:.3f} s"
    r = _to_host(got)
    np.testing.assert_array_equal(r["ip"], g["col"]("ip").astype(np.int32))
    np.testing.assert_array_equal(r["fjp"], g["col"]("fjp").astype(np.int32))
