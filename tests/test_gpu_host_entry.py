"""The host-buffer entry (xcg_correlate) against the device entry on the same
windows: it copies only the image rows the windows read, in bands that each
batch waits for, so its results must not depend on the location order, on
the part of the image the windows cover, or on what an earlier call left in
the context's image buffers.  Bar: every result field bit-identical to
xcg_correlate_device on fully resident images."""
import numpy as np
import pytest
import torch

import xcorr_gb300 as xg
from xcorr_gb300 import synth

pytestmark = pytest.mark.gpu


def _device(ctx, m, s, locs, strip_len, y_offset=0, astretcha=0.0):
    dev = torch.device("cuda", 0)
    dm, ds = torch.from_numpy(m).to(dev), torch.from_numpy(s).to(dev)
    dl = torch.from_numpy(np.ascontiguousarray(locs, np.int32)).to(dev)
    dr = torch.zeros((len(locs), xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    ctx.correlate_device(dm.data_ptr(), m.shape[1], m.shape[0], ds.data_ptr(), s.shape[1], s.shape[0],
                         dl.data_ptr(), len(locs), dr.data_ptr(), 0, y_offset=y_offset, astretcha=astretcha,
                         strip_len=strip_len)
    torch.cuda.synchronize()
    return np.frombuffer(dr.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)


def _same(a, b):
    assert a.tobytes() == b.tobytes()


@pytest.fixture(scope="module")
def pairs():
    p1 = synth.make_pair(synth.PairSpec(nx=1024, ny=3072, dx=1.3, dy=-2.2, noise_frac=0.1, seed=21))
    p2 = synth.make_pair(synth.PairSpec(nx=1024, ny=3072, dx=-0.6, dy=3.1, noise_frac=0.2, seed=22))
    return p1, p2


def test_sub_area_and_stale_buffers(pairs):
    (m1, s1), (m2, s2) = pairs
    full = xg.grid(1024, 3072, 6, 30, 64, 64)
    part = full[(full[:, 1] > 1200) & (full[:, 1] < 2000)]        # a band of strips in the middle
    with xg.Context(xg.params(64, 64), max_batch=96) as ctx:
        ctx.correlate(m1, s1, full, strip_len=6)                  # fills the image buffers with pair 1
        r = ctx.correlate(m2, s2, part, strip_len=6)              # reads only pair 2's rows it copies
        st = ctx.stats()
        d = _device(ctx, m2, s2, part, 6)
    _same(r, d)
    # the bytes it reports copying: the rows and columns of both images that
    # the 256 x 256 patches cover (no offsets here), the locations, the results
    y0, x0 = part[:, 1] - 128, part[:, 0] - 128
    rows = min(int(y0.max()) + 256, 3072) - max(int(y0.min()), 0)
    cols = min(int(x0.max()) + 256, 1024) - max(int(x0.min()), 0)
    assert st.h2d_bytes == 2 * rows * cols * 4 + part.nbytes
    assert st.h2d_bytes < m2.nbytes
    assert st.d2h_bytes == len(part) * xg.RESULT_DTYPE.itemsize


def test_location_order_and_shifted_slave(pairs):
    (m1, s1), _ = pairs
    locs = xg.grid(1024, 3072, 6, 30, 64, 64)
    rng = np.random.default_rng(5)
    strips = rng.permutation(len(locs) // 6)
    shuffled = np.concatenate([locs[6 * k:6 * k + 6] for k in strips])   # whole strips, any order
    for y_offset, ast in ((0, 0.0), (-37, 0.0), (12, 0.004)):
        with xg.Context(xg.params(64, 64), max_batch=64) as ctx:
            r = ctx.correlate(m1, s1, shuffled, 0, y_offset, ast, strip_len=6)
            st = ctx.stats()
            d = _device(ctx, m1, s1, shuffled, 6, y_offset, ast)
        assert st.batches >= 3
        _same(r, d)


def test_single_strip_job(pairs):
    (m1, s1), _ = pairs
    locs = xg.grid(1024, 3072, 6, 30, 64, 64)[-6:]                 # the last strip only
    with xg.Context(xg.params(64, 64)) as ctx:
        r = ctx.correlate(m1, s1, locs, strip_len=6)
        d = _device(ctx, m1, s1, locs, 6)
    _same(r, d)


def test_real_format_rows():
    """float32 real samples (-real): one 32-bit word per sample, like the
    int16 I/Q pairs, so the same row bands apply."""
    m, s = synth.make_pair(synth.PairSpec(nx=1024, ny=2048, dx=1.1, dy=-0.7, noise_frac=0.1, seed=23, real=True))
    locs = xg.grid(1024, 2048, 6, 20, 64, 64)
    part = locs[(locs[:, 1] > 500) & (locs[:, 1] < 1500)]
    p = xg.params(64, 64, fmt=1)
    with xg.Context(p, max_batch=48) as ctx:
        r = ctx.correlate(m, s, part, strip_len=6)
        d = _device(ctx, m, s, part, 6)
    _same(r, d)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_random_geometry(seed):
    """Seeded random jobs: window size, strip length (ragged last strip),
    location order by strip, slave offsets and azimuth stretch, batch size;
    every result field bit-identical to the device entry."""
    rng = np.random.default_rng(100 + seed)
    xs = int(rng.choice([32, 64]))
    nx, ny = int(rng.choice([768, 1024])), int(rng.choice([1536, 2048]))
    m, s = synth.make_pair(synth.PairSpec(nx=nx, ny=ny, dx=float(rng.uniform(-3, 3)), dy=float(rng.uniform(-3, 3)),
                                          noise_frac=0.1, seed=200 + seed))
    nxl = int(rng.integers(3, 9))
    locs = xg.grid(nx, ny, nxl, int(rng.integers(8, 20)), xs, xs)
    locs = locs[: len(locs) - int(rng.integers(0, nxl))]                 # ragged last strip
    nst = (len(locs) + nxl - 1) // nxl
    order = rng.permutation(nst)
    locs = np.concatenate([locs[k * nxl:(k + 1) * nxl] for k in order])
    y_offset = int(rng.integers(-20, 21))
    ast = float(rng.uniform(-2e-3, 2e-3))
    with xg.Context(xg.params(xs, xs), max_batch=int(rng.integers(16, 120))) as ctx:
        r = ctx.correlate(m, s, locs, 0, y_offset, ast, strip_len=nxl)
        d = _device(ctx, m, s, locs, nxl, y_offset, ast)
    _same(r, d)


def test_timeline_marks(pairs):
    """Timeline mode (xcg_set_profiling 2): the batches still overlap, the
    results are the same bits, and the marks come in the order each stream
    passed them: every image band, each batch's stages in order, then the
    join and the results."""
    (m1, s1), _ = pairs
    locs = xg.grid(1024, 3072, 16, 40, 64, 64)                    # 640 windows: two batches
    with xg.Context(xg.params(64, 64)) as ctx:
        plain = ctx.correlate(m1, s1, locs, strip_len=16)
        ctx.set_profiling(2)
        timed = ctx.correlate(m1, s1, locs, strip_len=16)
        tl = dict(ctx.timeline())
        st = ctx.stats()
    _same(plain, timed)
    assert st.batches == 2
    assert tl[1] == 0.0 and tl[3] >= tl[2] > 0.0
    bands = sorted(t for t in tl if 100 <= t < 1000)
    assert bands == list(range(100, 100 + len(bands))) and len(bands) >= 2
    assert all(tl[a] <= tl[b] for a, b in zip(bands, bands[1:]))          # one copy stream
    for b in range(st.batches):
        stages = [tl[1000 + 10 * b + k] for k in range(4)]
        assert stages == sorted(stages) and stages[-1] <= tl[2]


def test_batch_splits_same_bits(pairs):
    """Any number of batches per call (xcg_set_batches), alternating between
    the two scratch slots or four at a time in the half-slot lanes, gives the
    same bits on both entries; the host entry's automatic choice for a job of
    this size is four batches."""
    (m1, s1), _ = pairs
    locs = xg.grid(1024, 3072, 16, 60, 64, 64)                    # 960 windows, strips of 16
    with xg.Context(xg.params(64, 64)) as ctx:
        base = ctx.correlate(m1, s1, locs, strip_len=16)
        assert ctx.stats().batches == 4
        _same(_device(ctx, m1, s1, locs, 16), base)
        for nb, expect in ((1, 1), (2, 2), (3, 3), (5, 5), (8, 8)):
            ctx.set_batches(nb)
            r = ctx.correlate(m1, s1, locs, strip_len=16)
            assert ctx.stats().batches == expect
            _same(r, base)
            _same(_device(ctx, m1, s1, locs, 16), base)
