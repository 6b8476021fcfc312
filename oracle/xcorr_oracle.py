"""ctypes binding of the C oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker.  See xcorr_oracle.h for what the oracle restates.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

F32, F64 = 32, 64


class XoParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in
                ("npx", "npy", "nxc", "nyc", "nx_corr", "ny_corr", "xsearch", "ysearch",
                 "ri", "interp_flag", "ifc", "n2x", "n2y", "corr_mode")]


RESULT_DTYPE = np.dtype([
    ("xoff", "<f4"), ("yoff", "<f4"), ("xfrac", "<f4"), ("yfrac", "<f4"), ("corr", "<f4"),
    ("ip", "<i4"), ("jp", "<i4"), ("fip", "<i4"), ("fjp", "<i4"), ("flags", "<i4"),
    ("fmax", "<f4"),
    ("cmax", "<f8"), ("cave", "<f8"), ("cave_true", "<f8"), ("gamma", "<f8"),
    ("mean1", "<f8"), ("mean2", "<f8"), ("corr0n", "<f8"),
], align=True)

FLAG_OOB = 1
FLAG_NEXTREAD = 2


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.xo_run.restype = ctypes.c_int
        L.xo_run.argtypes = [ctypes.POINTER(XoParams), ctypes.c_int, ctypes.c_int,
                             ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                             ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                             ctypes.c_int, ctypes.c_int, ctypes.c_double,
                             ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                             ctypes.c_void_p]
        L.xo_range_interp_row.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.xo_prepare_patch.argtypes = [ctypes.POINTER(XoParams), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
        L.xo_surface.argtypes = [ctypes.POINTER(XoParams), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.xo_fine_surface.restype = ctypes.c_int
        L.xo_fine_surface.argtypes = [ctypes.POINTER(XoParams), ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_void_p]
        L.xo_time_surface.argtypes = [ctypes.POINTER(XoParams), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
        L.xo_argmax_ref.restype = ctypes.c_int64
        L.xo_argmax_ref.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


def params(xsearch=64, ysearch=64, ri=2, interp_flag=1, ifc=16, n2x=8, n2y=8, corr_mode=2) -> XoParams:
    """Parameters as parse_xcorr_input.c:67-86,139-158 derives them from xsearch/ysearch.
    corr_mode: 2 frequency domain (default), 0 -time, 1 -time4."""
    return XoParams(npx=4 * xsearch, npy=4 * ysearch, nxc=2 * xsearch, nyc=2 * ysearch,
                    nx_corr=2 * xsearch, ny_corr=2 * ysearch, xsearch=xsearch, ysearch=ysearch,
                    ri=ri, interp_flag=interp_flag, ifc=ifc, n2x=n2x, n2y=n2y, corr_mode=corr_mode)


def run(p: XoParams, master: np.ndarray, slave: np.ndarray, locs: np.ndarray,
        x_offset=0, y_offset=0, astretcha=0.0, precision=F32, strip_len=0, nthreads=0) -> np.ndarray:
    """Correlate every location.  master/slave: (ny, nx, 2) int16 or (ny, nx) float32."""
    fmt = 1 if master.dtype == np.float32 else 0
    master = np.ascontiguousarray(master)
    slave = np.ascontiguousarray(slave)
    locs = np.ascontiguousarray(locs, dtype=np.int32).reshape(-1, 2)
    out = np.zeros(len(locs), dtype=RESULT_DTYPE)
    rc = lib().xo_run(ctypes.byref(p), precision, fmt,
                      master.ctypes.data, master.shape[1], master.shape[0],
                      slave.ctypes.data, slave.shape[1], slave.shape[0],
                      int(x_offset), int(y_offset), float(astretcha),
                      locs.ctypes.data, len(locs), int(strip_len), int(nthreads), out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"xo_run failed: {rc}")
    return out


def range_interp_row(row: np.ndarray, ri: int, precision=F64) -> np.ndarray:
    row = np.ascontiguousarray(row, dtype=np.complex128)
    out = np.zeros_like(row)
    lib().xo_range_interp_row(precision, len(row), ri, row.ctypes.data, out.ctypes.data)
    return out


def prepare_patch(p: XoParams, patch: np.ndarray, slave: bool, precision=F32):
    """patch: (npy, npx) complex64.  Returns (amplitude float32, mean, ints int32)."""
    patch = np.ascontiguousarray(patch, dtype=np.complex64)
    amp = np.zeros((p.npy, p.npx), np.float32)
    ints = np.zeros((p.npy, p.npx), np.int32)
    mean = ctypes.c_double()
    lib().xo_prepare_patch(ctypes.byref(p), precision, int(slave), patch.ctypes.data, amp.ctypes.data,
                           ctypes.byref(mean), ints.ctypes.data)
    return amp, mean.value, ints


def time_surface(p: XoParams, i1: np.ndarray, i2: np.ndarray):
    """-time / -time4 (p.corr_mode 0 / 1) full-search surface of one window's
    (int) patches (npy, npx) and do_time_corr's peak as a result record."""
    i1 = np.ascontiguousarray(i1, dtype=np.int32)
    i2 = np.ascontiguousarray(i2, dtype=np.int32)
    corr = np.zeros((p.nyc, p.nxc), np.float64)
    r = np.zeros(1, dtype=RESULT_DTYPE)
    lib().xo_time_surface(ctypes.byref(p), i1.ctypes.data, i2.ctypes.data, corr.ctypes.data, r.ctypes.data)
    return corr, r[0]


def surface(p: XoParams, pm: np.ndarray, ps: np.ndarray, precision=F32):
    pm = np.ascontiguousarray(pm, dtype=np.complex64)
    ps = np.ascontiguousarray(ps, dtype=np.complex64)
    corr = np.zeros((p.nyc, p.nxc), np.float64)
    m1, m2 = ctypes.c_double(), ctypes.c_double()
    lib().xo_surface(ctypes.byref(p), precision, pm.ctypes.data, ps.ctypes.data, corr.ctypes.data,
                     ctypes.byref(m1), ctypes.byref(m2))
    return corr, m1.value, m2.value


def argmax_ref(x: np.ndarray):
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    v = ctypes.c_double()
    i = lib().xo_argmax_ref(x.ctypes.data, len(x), ctypes.byref(v))
    return int(i), v.value


def output_offsets(res: np.ndarray, ri: int, x_offset: int, y_offset: int, locs_y: np.ndarray,
                   astretcha: float):
    """Offsets as print_results writes them (print_results.c:30-38), in float32."""
    f = np.float32
    ishft = np.trunc(locs_y.astype(np.float64) * astretcha).astype(np.int32)
    xo = (res["xoff"].astype(f) / f(ri)) - (res["xfrac"].astype(f) / f(ri)) + f(x_offset)
    yo = res["yoff"].astype(f) - res["yfrac"].astype(f) + f(y_offset) + ishft.astype(f)
    return xo.astype(f), yo.astype(f)


def fine_surface(p: XoParams, master, slave, x, y, x_offset=0, y_offset=0, astretcha=0.0, precision=F64):
    """The interpolated real surface (ny2 x nx2) of one location, and its result."""
    fmt = 1 if master.dtype == np.float32 else 0
    master = np.ascontiguousarray(master)
    slave = np.ascontiguousarray(slave)
    ny2, nx2 = p.n2y * p.ifc, p.n2x * p.ifc
    re = np.zeros((ny2, nx2), np.float64)
    r = np.zeros(1, dtype=RESULT_DTYPE)
    rc = lib().xo_fine_surface(ctypes.byref(p), precision, fmt, master.ctypes.data, master.shape[1], master.shape[0],
                               slave.ctypes.data, slave.shape[1], slave.shape[0], int(x_offset), int(y_offset),
                               float(astretcha), int(x), int(y), re.ctypes.data, r.ctypes.data)
    if rc != 0:
        raise RuntimeError("xo_fine_surface failed")
    return re, r[0]


def near_tie(p: XoParams, master, slave, x, y, a, b, x_offset=0, y_offset=0, astretcha=0.0, rel=1e-5):
    """True when fine peaks a and b (row, col) are neighbouring cells whose FP64
    interpolated values agree within `rel` of the peak value: a tie that FP32
    rounding in either implementation can break either way."""
    if abs(a[0] - b[0]) > 1 or abs(a[1] - b[1]) > 1:
        return False
    re, _ = fine_surface(p, master, slave, x, y, x_offset, y_offset, astretcha)
    va, vb = re[a[0], a[1]], re[b[0], b[1]]
    return abs(va - vb) <= rel * max(abs(va), abs(vb))
