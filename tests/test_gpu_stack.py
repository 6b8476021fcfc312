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
    for it, a in zip(items, alone):
        if it["nxl"] <= 7:
            _same(_host(it["dr"]), a)
    assert len(cache.read_text().splitlines()) >= 1 + 4
    st.close()
