"""Helpers shared by the golden-vector tests: load a reference record,
regenerate its inputs, and derive the reference's parameters and location grid
(set_defaults / parse_command_line / get_locations restated for the tests)."""
import gzip
import json
import os

import numpy as np

from cases import CASES
from xcorr_gb300 import synth

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with gzip.open(os.path.join(GOLDEN_DIR, f"ref_{name}.json.gz"), "rt") as f:
        g = json.load(f)
    cols = {c: i for i, c in enumerate(g["dump_cols"])}
    g["D"] = np.array(g["dump"], dtype=np.float64)
    g["col"] = lambda c: g["D"][:, cols[c]]
    return g


def parse_flags(flags):
    """The options of parse_xcorr_input.c:99-182 that the golden cases use."""
    d = dict(nxl=16, nyl=32, xsearch=64, ysearch=64, ri=2, interp_flag=1, ifc=16, real=False, noshift=False)
    it = iter(flags)
    for f in it:
        if f == "-nx": d["nxl"] = int(next(it))
        elif f == "-ny": d["nyl"] = int(next(it))
        elif f == "-xsearch": d["xsearch"] = int(next(it))
        elif f == "-ysearch": d["ysearch"] = int(next(it))
        elif f == "-range_interp": d["ri"] = int(next(it))
        elif f == "-norange": d["ri"] = 1
        elif f == "-interp": d["ifc"] = int(next(it)); d["interp_flag"] = 1
        elif f == "-nointerp": d["interp_flag"] = 0
        elif f == "-real": d["real"] = True
        elif f == "-noshift": d["noshift"] = True
        else: raise ValueError(f)
    return d


def grid(m_nx, m_ny, nxl, nyl, xsearch, ysearch):
    """get_locations.c:21-40 with npx=4*xsearch, nx_corr=2*xsearch."""
    npx, npy, nxc_, nyc_ = 4 * xsearch, 4 * ysearch, 2 * xsearch, 2 * ysearch
    x_inc = (m_nx - 2 * (xsearch + nxc_)) // (nxl + 3)
    y_inc = (m_ny - 2 * (ysearch + nyc_)) // (nyl + 1)
    return np.array([(npx + i * x_inc, npy + j * y_inc)
                     for j in range(1, nyl + 1) for i in range(2, nxl + 2)], np.int32)


def case_inputs(name, g=None):
    """(master, slave, locs, flags-dict, x_offset, y_offset, astretcha) for a golden case."""
    g = g or load(name)
    m, s = synth.make_pair(CASES[name]["spec"])
    d = parse_flags(g["flags"])
    locs = grid(m.shape[1], m.shape[0], d["nxl"], d["nyl"], d["xsearch"], d["ysearch"])
    xoff, yoff = (0, 0) if d["noshift"] else (g["rshift"], g["ashift"])
    ast = (g["prf_slave"] - g["prf_master"]) / g["prf_master"]
    return m, s, locs, d, xoff, yoff, ast


def cut_patches(m, s, x, y, npx, npy, x_offset=0, y_offset=0, astretcha=0.0):
    """The master and slave patches of location (x, y) as complex64 (npy, npx)
    arrays, zero outside the images (xcorr.cu:330-338 on the lines
    read_xcorr_data.c:52-85 reads; the slave row origin adds y_offset and
    (int)(y * astretcha))."""
    def cut(img, x0, y0):
        out = np.zeros((npy, npx), np.complex64)
        ny, nx = img.shape[:2]
        ya, yb, xa, xb = max(y0, 0), min(y0 + npy, ny), max(x0, 0), min(x0 + npx, nx)
        if ya < yb and xa < xb:
            blk = img[ya:yb, xa:xb]
            z = blk.astype(np.float32) if blk.ndim == 2 else blk[..., 0].astype(np.float32) + 1j * blk[..., 1].astype(np.float32)
            out[ya - y0:yb - y0, xa - x0:xb - x0] = z
        return out
    ishft = int(y * astretcha)
    return (cut(m, x - npx // 2, y - npy // 2),
            cut(s, x + x_offset - npx // 2, y + y_offset + ishft - npy // 2))
