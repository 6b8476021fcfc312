"""Run the reference's -time / -time4 correlation (do_time_corr with
calc_time_corr / calc_time_corr_hat, do_time_int_xcorr.cu:30-189) on windows
of two golden cases and record what it computes.

The reference's GPU program never fills the integer patches these host
functions read (xcorr.cu:364-368), so its program cannot be run in these
modes; oracle/_ref/ref_time_probe (built by oracle/ref/build_ref.sh from the
reference sources) drives the functions themselves.  Their inputs are the
(int) demeaned amplitudes of each window's range-interpolated master and
masked slave patch as the oracle prepares them (FP32, as the frequency path
does; the oracle's preparation is pinned to the reference by the golden
means and correlations).  Per window and mode the record holds the SHA-256
of both integer patches, the SHA-256 of the reference's float64 surface, 64
sampled surface values, the surface maximum and the struct locs fields the
reference sets (xoff, yoff, corr).  Runs on the CPU.

usage: python tests/golden/make_ref_time.py --out DIR
"""
import argparse
import gzip
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
for p in (_HERE, os.path.join(_HERE, ".."), os.path.join(_HERE, "..", "..", "oracle"),
          os.path.join(_HERE, "..", "..", "gmtsar-gpu_gb300", "python")):
    sys.path.insert(0, p)
import golden_util as gu  # noqa: E402
import xcorr_oracle as xo  # noqa: E402

PROBE = os.path.join(_HERE, "..", "..", "oracle", "_ref", "ref_time_probe")
# (golden case, windows): four 64x64 windows, one 128x128 window, one window
# whose master patch is all zero (denominator zero: corr 0)
WINDOWS = {"xs32": [0, 1, 9, 20], "cfg1": [0], "zeroband": [8]}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def int_patches(name, w):
    g = gu.load(name)
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs(name, g)
    x, y = (int(v) for v in locs[w])
    p = xo.params(d["xsearch"], d["ysearch"], d["ri"])
    pm, ps = gu.cut_patches(m, s, x, y, p.npx, p.npy, xoff, yoff, ast)
    i1 = xo.prepare_patch(p, pm, False, xo.F32)[2]
    i2 = xo.prepare_patch(p, ps, True, xo.F32)[2]
    return d, (x, y), i1, i2


def sample_index(nyc, nxc):
    """64 lags spread over the surface, the same in every record."""
    rng = np.random.default_rng(7)
    return np.sort(rng.choice(nyc * nxc, 64, replace=False))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    recs = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, wins in WINDOWS.items():
            for w in wins:
                d, (x, y), i1, i2 = int_patches(name, w)
                f1, f2, fo = (os.path.join(tmp, f) for f in ("i1.bin", "i2.bin", "out.bin"))
                i1.tofile(f1)
                i2.tofile(f2)
                for mode in (0, 1):
                    subprocess.run([PROBE, str(d["xsearch"]), str(d["ysearch"]), str(mode), f1, f2, fo], check=True,
                                   stderr=subprocess.DEVNULL)   # calc_time_corr_hat prints per zero lag
                    nyc, nxc = 2 * d["ysearch"], 2 * d["xsearch"]
                    raw = open(fo, "rb").read()
                    surf = np.frombuffer(raw[:nyc * nxc * 8], np.float64).reshape(nyc, nxc)
                    xoff, yoff, corr = np.frombuffer(raw[nyc * nxc * 8:], np.float32)
                    idx = sample_index(nyc, nxc)
                    recs.append(dict(case=name, window=w, x=x, y=y, mode=mode, i1_sha256=sha(i1), i2_sha256=sha(i2),
                                     surface_sha256=sha(surf), sample_index=idx.tolist(),
                                     sample_value=[float(v) for v in surf.ravel()[idx]],
                                     surface_max=float(np.abs(surf).max()),
                                     xoff=float(xoff), yoff=float(yoff), corr=float(corr)))
                    print(name, w, mode, recs[-1]["xoff"], recs[-1]["yoff"], recs[-1]["corr"])
    with gzip.open(os.path.join(a.out, "ref_time.json.gz"), "wt") as f:
        json.dump({"generator": "tests/golden/make_ref_time.py", "records": recs}, f)


if __name__ == "__main__":
    main()
