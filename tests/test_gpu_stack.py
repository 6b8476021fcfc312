"""Stack scheduler on the GPU: a stack of pairs with mixed window sizes,
image sizes, shifts and strip lengths must give, window for window, the same
results as correlating each pair alone; graph capture and replay, the batch
autotuner and strip-preserving batch splits must not change them."""
import os

import numpy as np
import pytest

import xcorr_gb300 as xg
from xcorr_gb300 import synth

pytestmark = pytest.mark.gpu

STACK = [  # (nx, ny, dx, dy, xsearch, ysearch, nxl, nyl, x_offset, y_offset, astretcha)
    (1024, 1024, 1.3, -2.2, 32, 32, 5, 3, 0, 0, 0.0),
    (1536, 2048, -3.4, 4.1, 64, 64, 4, 2, 2, -3, 1e-3),
    (1024, 1536, 0.4, 0.9, 32, 64, 3, 4, 0, 0, 0.0),
    (1280, 1280, 2.6, -0.7, 32, 32, 9, 2, 0, 0, 0.0),
    (2048, 1024, -1.1, 1.8, 64, 32, 2, 3, 1, 1, 0.0),
]


def _setup(torch):
    dev = torch.device("cuda", 0)
    items = []
    for i, (nx, ny, dx, dy, xs, ys, nxl, nyl, xo, yo, ast) in enumerate(STACK):
        m, s = synth.make_pair(synth.PairSpec(nx=nx, ny=ny, dx=dx, dy=dy, noise_frac=0.2, seed=100 + i))
        locs = xg.grid(nx, ny, nxl, nyl, xs, ys)
        items.append(dict(m=m, s=s, locs=locs, xs=xs, ys=ys, nxl=nxl, xo=xo, yo=yo, ast=ast,
                          dm=torch.from_numpy(m).to(dev), ds=torch.from_numpy(s).to(dev),
                          dr=torch.zeros((len(locs), xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)))
    return items


def _pairs(items):
    out = []
    for it in items:
        out.append(xg.Pair(d_master=it["dm"].data_ptr(), m_nx=it["m"].shape[1], m_ny=it["m"].shape[0],
                           d_slave=it["ds"].data_ptr(), s_nx=it["s"].shape[1], s_ny=it["s"].shape[0],
                           x_offset=it["xo"], y_offset=it["yo"], astretcha=it["ast"],
                           locs=it["locs"].ctypes.data, nlocs=len(it["locs"]), strip_len=it["nxl"],
                           xsearch=it["xs"], ysearch=it["ys"], d_results=it["dr"].data_ptr()))
    return out


def _host(t):
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)


def _alone(it):
    with xg.Context(xg.params(it["xs"], it["ys"])) as ctx:
        return ctx.correlate(it["m"], it["s"], it["locs"], it["xo"], it["yo"], it["ast"], strip_len=it["nxl"])


def _same(a, b):
    for k in RESULT_KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


RESULT_KEYS = ("ip", "jp", "fip", "fjp", "flags", "xoff", "yoff", "xfrac", "yfrac", "corr", "gamma", "cmax", "cave")


def test_stack_equals_pairs_alone_and_graph_replay():
    torch = pytest.importorskip("torch")
    items = _setup(torch)
    alone = [_alone(it) for it in items]
    st = xg.Stack(xg.params())
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        st.run(_pairs(items), stream.cuda_stream)
    stream.synchronize()
    for it, a in zip(items, alone):
        _same(_host(it["dr"]), a)
    s = st.stats()
    assert s.buckets == 4 and s.windows == sum(len(it["locs"]) for it in items)
    # graph: capture, then replay into cleared result arrays
    st.set_graph(True)
    for rep in range(3):
        for it in items:
            it["dr"].zero_()
        torch.cuda.synchronize()
        st.run(_pairs(items), stream.cuda_stream)
        stream.synchronize()
        for it, a in zip(items, alone):
            _same(_host(it["dr"]), a)
    assert st.stats().graph_replays == 2
    st.close()


def test_autotune_and_split_strips(tmp_path, monkeypatch):
    torch = pytest.importorskip("torch")
    items = _setup(torch)
    alone = [_alone(it) for it in items]
    # a cache entry forces 7 windows per batch for the 128x128 patch bucket:
    # strips of 5 and 3 end inside batches, strips of 9 are split
    cache = tmp_path / "tune.txt"
    cache.write_text("128 128 2 16 7\n")
    monkeypatch.setenv("XCG_TUNE_CACHE", str(cache))
    st = xg.Stack(xg.params())
    st.run(_pairs(items), 0)
    torch.cuda.synchronize()
    assert 7 in list(st.stats().bucket_batch)
    for it, a in zip(items, alone):
        got = _host(it["dr"])
        if it["nxl"] <= 7:
            _same(got, a)
        else:   # a split strip loses only the next-window read at the split
            for k in ("ip", "jp", "corr", "gamma"):
                np.testing.assert_array_equal(got[k], a[k], err_msg=k)
    st.autotune(_pairs(items), 0)
    torch.cuda.synchronize()
    for it in items:
        it["dr"].zero_()
    st.run(_pairs(items), 0)
    torch.cuda.synchronize()
    # the tuner may pick one row stage per window for a bucket: the same
    # peaks and offsets, the correlation within FP32 rounding
    for it, a in zip(items, alone):
        if it["nxl"] <= 7:
            got = _host(it["dr"])
            for k in ("ip", "jp", "fip", "fjp", "flags", "xoff", "yoff", "xfrac", "yfrac"):
                np.testing.assert_array_equal(got[k], a[k], err_msg=k)
            assert np.max(np.abs(got["gamma"] / a["gamma"] - 1)) < 1e-5
    lines = cache.read_text().splitlines()
    assert len(lines) >= 1 + 4 and all(len(l.split()) == 8 for l in lines[1:])
    s = st.stats()
    assert all(0 <= s.bucket_cols_cfg[i] <= 2 and 0 <= s.bucket_peak_cfg[i] <= 2 for i in range(s.buckets))
    st.close()


def test_stack_every_bucket_against_oracle():
    """One stack holding windows of 32, 64, 128 and 256 (xsearch 16 to 128,
    one bucket each, pairs of different sizes, offsets and stretch): every
    window against the oracle's FP32 restatement of the reference path,
    integer and subpixel peaks identical, correlation within 1e-4."""
    torch = pytest.importorskip("torch")
    import xcorr_oracle as xo
    dev = torch.device("cuda", 0)
    spec = [(768, 768, 1.6, -0.8, 16, 16, 6, 4, 0, 0, 0.0),
            (1024, 1024, -2.2, 1.3, 32, 32, 4, 3, 3, -2, 5e-4),
            (1536, 1536, 0.7, 2.6, 64, 64, 3, 2, 0, 0, 0.0),
            (2560, 2560, -1.9, -3.3, 128, 128, 2, 2, 0, 0, 0.0)]
    items = []
    for i, (nx, ny, dx, dy, xs, ys, nxl, nyl, xoff, yoff, ast) in enumerate(spec):
        m, s = synth.make_pair(synth.PairSpec(nx=nx, ny=ny, dx=dx, dy=dy, noise_frac=0.1, seed=300 + i))
        locs = xg.grid(nx, ny, nxl, nyl, xs, ys)
        items.append(dict(m=m, s=s, locs=locs, xs=xs, ys=ys, nxl=nxl, xo=xoff, yo=yoff, ast=ast,
                          dm=torch.from_numpy(m).to(dev), ds=torch.from_numpy(s).to(dev),
                          dr=torch.zeros((len(locs), xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)))
    st = xg.Stack(xg.params())
    st.run(_pairs(items), 0)
    torch.cuda.synchronize()
    assert st.stats().buckets == 4
    for it in items:
        got = _host(it["dr"])
        o = xo.run(xo.params(it["xs"], it["ys"]), it["m"], it["s"], it["locs"], it["xo"], it["yo"], it["ast"],
                   precision=xo.F32, strip_len=it["nxl"])
        for k in ("ip", "jp", "fip", "fjp", "flags"):
            np.testing.assert_array_equal(got[k], o[k], err_msg=f"window {2 * it['xs']}: {k}")
        rel = np.abs(got["gamma"] - o["gamma"]) / np.abs(o["gamma"])
        assert rel.max() < 1e-4, (it["xs"], rel.max())
    st.close()


@pytest.mark.parametrize("cols_cfg,peak_cfg", [(0, 1), (1, 0), (2, 1), (1, 1), (0, 2), (2, 2)])
def test_tuned_launch_shapes_give_identical_results(tmp_path, monkeypatch, cols_cfg, peak_cfg):
    """Every per-window launch shape the autotuner chooses between (256-thread
    column CTAs, one cp.async staging group, one peak CTA per SM fewer, 512
    peak threads per window) computes the same transforms in the same order:
    results bit-identical to a context with one row stage per window."""
    torch = pytest.importorskip("torch")
    items = _setup(torch)
    alone = []
    for it in items:
        with xg.Context(xg.params(it["xs"], it["ys"])) as ctx:
            ctx.set_row_sharing(False)
            alone.append(ctx.correlate(it["m"], it["s"], it["locs"], it["xo"], it["yo"], it["ast"],
                                       strip_len=it["nxl"]))
    cache = tmp_path / "tune.txt"
    cache.write_text("".join(f"{4 * xs} {4 * ys} 2 16 0 {cols_cfg} {peak_cfg} 0\n"
                             for xs, ys in {(it["xs"], it["ys"]) for it in items}))
    monkeypatch.setenv("XCG_TUNE_CACHE", str(cache))
    st = xg.Stack(xg.params())
    st.run(_pairs(items), 0)
    torch.cuda.synchronize()
    s = st.stats()
    assert [s.bucket_cols_cfg[i] for i in range(s.buckets)] == [cols_cfg] * s.buckets
    assert [s.bucket_peak_cfg[i] for i in range(s.buckets)] == [peak_cfg] * s.buckets
    assert [s.bucket_row_sharing[i] for i in range(s.buckets)] == [0] * s.buckets
    for it, a in zip(items, alone):
        _same(_host(it["dr"]), a)
    st.close()
