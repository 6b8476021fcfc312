"""ctypes binding of libxcorr_gb300.so (the C ABI in include/xcorr_gb300.h).

This module only marshals arguments: every computation runs in the CUDA
library.  Loading fails loudly when the library is missing; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB_PATH = os.path.join(_PKG, "lib", "libxcorr_gb300.so")

XCG_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "out of memory",
          5: "no usable CUDA device", 6: "size exceeds a fixed limit"}
FLAG_OOB = 1
FLAG_NEXTREAD = 2

# every entry point include/xcorr_gb300.h declares
EXPORTS = ("xcg_status_string", "xcg_last_error", "xcg_default_params", "xcg_create", "xcg_destroy",
           "xcg_correlate", "xcg_correlate_device", "xcg_correlate_device_noalloc", "xcg_set_profiling",
           "xcg_get_stats", "xcg_stack_create", "xcg_stack_destroy", "xcg_stack_run", "xcg_stack_set_graph",
           "xcg_stack_autotune", "xcg_stack_get_stats", "xcg_set_features", "xcg_refiner_create",
           "xcg_refiner_destroy", "xcg_refiner_set_params", "xcg_refiner_get_params", "xcg_refiner_forward",
           "xcg_refiner_gradient", "xcg_refiner_train_step", "xcg_correlate_device_refined",
           "xcg_fit_offsets", "xcg_tc_gemm_check", "xcg_set_dft_form", "xcg_debug_inject_stage_timeout",
           "xcg_fp32_fma_rate", "xcg_set_row_sharing", "xcg_set_launch_shapes", "xcg_set_batches")
REFINER_NPARAM = 37507
FLAG_REFINED = 4
FLAG_STAGE_TIMEOUT = 8
NOALLOC_SCRATCH_BYTES = 32 << 20


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ("xsearch", "ysearch", "nx_corr", "ny_corr", "ri", "interp_flag", "interp_factor",
                 "n2x", "n2y", "format", "corr_mode")]


class Loc(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int32), ("y", ctypes.c_int32)]


RESULT_DTYPE = np.dtype([
    ("xoff", "<f4"), ("yoff", "<f4"), ("xfrac", "<f4"), ("yfrac", "<f4"), ("corr", "<f4"),
    ("ip", "<i4"), ("jp", "<i4"), ("fip", "<i4"), ("fjp", "<i4"), ("flags", "<i4"),
    ("fmax", "<f4"),
    ("cmax", "<f8"), ("cave", "<f8"), ("cave_true", "<f8"), ("gamma", "<f8"),
    ("mean1", "<f8"), ("mean2", "<f8"), ("corr0n", "<f8"),
], align=True)


class Stats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int64), ("batches", ctypes.c_int32), ("batch_windows", ctypes.c_int32),
                ("kernel_ms", ctypes.c_double * 8), ("scratch_bytes", ctypes.c_size_t),
                ("nkernels", ctypes.c_int32), ("pad", ctypes.c_int32), ("row_chunks", ctypes.c_int64),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64), ("host_enqueue_ms", ctypes.c_double),
                ("timeline_n", ctypes.c_int32), ("timeline_tag", ctypes.c_int32 * 64), ("timeline_ms", ctypes.c_float * 64)]


KERNEL_NAMES = ("k_rows", "k_cols", "k_peak", "k_subpix")
# launch slots with shared row segments: the planner and row kernel time together in slot 0
RC_KERNEL_NAMES = ("k_segrows", "k_cols_rc", "k_peak", "k_subpix")
TC_KERNEL_NAMES = ("k_rows", "k_tc_rows", "k_tc_cols", "k_tc_inv", "k_peak", "k_subpix")


class FitAxis(ctypes.Structure):
    """xcg_fit_axis: offset = shift + stretch*x + a_stretch*y."""
    _fields_ = [("shift", ctypes.c_double), ("stretch", ctypes.c_double), ("a_stretch", ctypes.c_double),
                ("sub_int", ctypes.c_double), ("rms", ctypes.c_double), ("weight", ctypes.c_double),
                ("ishift", ctypes.c_int32), ("npts", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Fit(ctypes.Structure):
    _fields_ = [("range", FitAxis), ("azimuth", FitAxis)]


class Pair(ctypes.Structure):
    """xcg_pair: one pair of a stack (device images and results, host locations)."""
    _fields_ = [("d_master", ctypes.c_void_p), ("m_nx", ctypes.c_int32), ("m_ny", ctypes.c_int32),
                ("d_slave", ctypes.c_void_p), ("s_nx", ctypes.c_int32), ("s_ny", ctypes.c_int32),
                ("x_offset", ctypes.c_int32), ("y_offset", ctypes.c_int32), ("astretcha", ctypes.c_double),
                ("locs", ctypes.c_void_p), ("nlocs", ctypes.c_int32), ("strip_len", ctypes.c_int32),
                ("xsearch", ctypes.c_int32), ("ysearch", ctypes.c_int32), ("d_results", ctypes.c_void_p),
                ("d_features", ctypes.c_void_p)]


class StackStats(ctypes.Structure):
    _fields_ = [("windows", ctypes.c_int64), ("launches", ctypes.c_int64), ("graph_replays", ctypes.c_int64),
                ("last_graph_launches", ctypes.c_int64), ("batches", ctypes.c_int32),
                ("last_graph_batches", ctypes.c_int32), ("buckets", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("bucket_npx", ctypes.c_int32 * 8), ("bucket_npy", ctypes.c_int32 * 8),
                ("bucket_batch", ctypes.c_int32 * 8), ("bucket_cols_cfg", ctypes.c_int32 * 8),
                ("bucket_peak_cfg", ctypes.c_int32 * 8), ("bucket_row_sharing", ctypes.c_int32 * 8)]

_lib = None


class XcgError(RuntimeError):
    pass


def load(path: str | None = None):
    """Load the CUDA library (build it first with gmtsar-gpu_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise XcgError(f"libxcorr_gb300.so not found at {path}; run gmtsar-gpu_gb300/build.py")
    L = ctypes.CDLL(path)
    L.xcg_status_string.restype = ctypes.c_char_p
    L.xcg_status_string.argtypes = [ctypes.c_int]
    L.xcg_last_error.restype = ctypes.c_char_p
    L.xcg_default_params.argtypes = [ctypes.POINTER(Params)]
    L.xcg_create.restype = ctypes.c_int
    L.xcg_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
    L.xcg_destroy.argtypes = [ctypes.c_void_p]
    L.xcg_correlate.restype = ctypes.c_int
    L.xcg_correlate.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
    L.xcg_correlate_device.restype = ctypes.c_int
    L.xcg_correlate_device.argtypes = L.xcg_correlate.argtypes + [ctypes.c_void_p]
    L.xcg_correlate_device_noalloc.restype = ctypes.c_int
    L.xcg_correlate_device_noalloc.argtypes = [ctypes.POINTER(Params)] + L.xcg_correlate.argtypes[1:] + [ctypes.c_void_p]
    L.xcg_stack_create.restype = ctypes.c_int
    L.xcg_stack_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
    L.xcg_stack_destroy.argtypes = [ctypes.c_void_p]
    L.xcg_stack_run.restype = ctypes.c_int
    L.xcg_stack_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(Pair), ctypes.c_int32, ctypes.c_void_p]
    L.xcg_stack_autotune.restype = ctypes.c_int
    L.xcg_stack_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(Pair), ctypes.c_int32, ctypes.c_void_p]
    L.xcg_stack_set_graph.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.xcg_stack_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(StackStats)]
    L.xcg_set_features.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.xcg_refiner_create.restype = ctypes.c_int
    L.xcg_refiner_create.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
    L.xcg_refiner_destroy.argtypes = [ctypes.c_void_p]
    for fn in ("xcg_refiner_set_params", "xcg_refiner_get_params"):
        getattr(L, fn).restype = ctypes.c_int
        getattr(L, fn).argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.xcg_refiner_forward.restype = ctypes.c_int
    L.xcg_refiner_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                      ctypes.c_int32, ctypes.c_void_p]
    L.xcg_refiner_gradient.restype = ctypes.c_int
    L.xcg_refiner_gradient.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
                                       ctypes.c_void_p]
    L.xcg_refiner_train_step.restype = ctypes.c_int
    L.xcg_refiner_train_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                         ctypes.c_float, ctypes.c_void_p]
    L.xcg_correlate_device_refined.restype = ctypes.c_int
    L.xcg_correlate_device_refined.argtypes = ([ctypes.c_void_p, ctypes.c_void_p] + L.xcg_correlate.argtypes[1:]
                                               + [ctypes.c_float, ctypes.c_float, ctypes.c_void_p])
    L.xcg_fit_offsets.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_double, ctypes.c_float, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    L.xcg_tc_gemm_check.argtypes = [ctypes.c_int32] * 4 + [ctypes.c_void_p] * 4
    L.xcg_set_dft_form.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.xcg_debug_inject_stage_timeout.argtypes = [ctypes.c_void_p]
    L.xcg_set_row_sharing.restype = ctypes.c_int
    L.xcg_set_row_sharing.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.xcg_set_launch_shapes.restype = ctypes.c_int
    L.xcg_set_launch_shapes.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]
    L.xcg_set_batches.restype = ctypes.c_int
    L.xcg_set_batches.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.xcg_fp32_fma_rate.restype = ctypes.c_int
    L.xcg_fp32_fma_rate.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
    L.xcg_set_profiling.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.xcg_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats)]
    _lib = L
    return L


def _check(rc):
    if rc != XCG_OK:
        L = load()
        raise XcgError(f"{L.xcg_status_string(rc).decode()}: {L.xcg_last_error().decode()}")


def params(xsearch=64, ysearch=64, ri=2, interp_flag=1, interp_factor=16, fmt=0, corr_mode=2) -> Params:
    """Parameters derived the way parse_xcorr_input.c:139-158 couples them.
    corr_mode: 2 frequency domain (default), 0 -time, 1 -time4."""
    return Params(xsearch=xsearch, ysearch=ysearch, nx_corr=2 * xsearch, ny_corr=2 * ysearch, ri=ri,
                  interp_flag=interp_flag, interp_factor=interp_factor, n2x=8, n2y=8, format=fmt,
                  corr_mode=corr_mode)


class Context:
    """One correlation context (xcg_create ... xcg_destroy)."""

    def __init__(self, p: Params, device: int = 0, max_batch: int = 0):
        self._L = load()
        self.params = p
        h = ctypes.c_void_p()
        _check(self._L.xcg_create(ctypes.byref(p), device, max_batch, ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            self._L.xcg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_profiling(self, on):
        """True/1: events around every launch, batches in order (kernel_ms); 2: timeline marks with the
        batches overlapping (timeline()); False/0: off."""
        self._L.xcg_set_profiling(self._h, 2 if on == 2 else (1 if on else 0))

    def timeline(self):
        """[(tag, ms)] of the last call in timeline mode (tags: include/xcorr_gb300.h, xcg_stats)."""
        st = self.stats()
        return [(int(st.timeline_tag[i]), float(st.timeline_ms[i])) for i in range(st.timeline_n)]

    def set_dft_form(self, form: int):
        """0: FP32 SIMT FFTs (default); 1: split-FP16 tensor-core DFTs (precision form)."""
        _check(self._L.xcg_set_dft_form(self._h, int(form)))

    def set_row_sharing(self, on: bool):
        """Row stage once per shared image row segment (default) or once per window."""
        _check(self._L.xcg_set_row_sharing(self._h, 1 if on else 0))

    def set_launch_shapes(self, cols_cfg: int, peak_cfg: int = 0):
        """Column- and peak-stage launch shapes (xcg_set_launch_shapes); the results do not depend on them."""
        _check(self._L.xcg_set_launch_shapes(self._h, int(cols_cfg), int(peak_cfg)))

    def set_batches(self, batches: int):
        """Batches per call, 0 automatic (xcg_set_batches); the results do not depend on it."""
        _check(self._L.xcg_set_batches(self._h, int(batches)))

    def inject_stage_timeout(self):
        """The next precision-form call behaves as if a tensor-core wait had run out (error-path tests)."""
        self._L.xcg_debug_inject_stage_timeout(self._h)

    def stats(self) -> Stats:
        s = Stats()
        self._L.xcg_get_stats(self._h, ctypes.byref(s))
        return s

    def correlate(self, master: np.ndarray, slave: np.ndarray, locs: np.ndarray, x_offset=0, y_offset=0,
                  astretcha=0.0, strip_len=0) -> np.ndarray:
        """Host arrays in, host results out.  master/slave: (ny, nx, 2) int16 or (ny, nx) float32."""
        master = np.ascontiguousarray(master)
        slave = np.ascontiguousarray(slave)
        for name, a in (("master", master), ("slave", slave)):
            if self.params.format == 0 and (a.dtype != np.int16 or a.ndim != 3 or a.shape[2] != 2):
                raise ValueError(f"{name}: complex int16 images are (ny, nx, 2) int16 arrays, got {a.dtype} {a.shape}")
            if self.params.format == 1 and (a.dtype != np.float32 or a.ndim != 2):
                raise ValueError(f"{name}: -real images are (ny, nx) float32 arrays, got {a.dtype} {a.shape}")
        locs = np.ascontiguousarray(locs, dtype=np.int32).reshape(-1, 2)
        out = np.empty(len(locs), dtype=RESULT_DTYPE)        # the call writes every record
        _check(self._L.xcg_correlate(self._h, master.ctypes.data, master.shape[1], master.shape[0],
                                     slave.ctypes.data, slave.shape[1], slave.shape[0],
                                     int(x_offset), int(y_offset), float(astretcha),
                                     locs.ctypes.data, len(locs), int(strip_len), out.ctypes.data))
        return out

    def set_features(self, d_features: int | None):
        """Also write each window's normalised 9x9 peak neighbourhood (device [nlocs][81])."""
        self._L.xcg_set_features(self._h, d_features)

    def correlate_device_refined(self, refiner: "Refiner", d_master: int, m_nx: int, m_ny: int, d_slave: int,
                                 s_nx: int, s_ny: int, d_locs: int, nlocs: int, d_results: int, stream: int = 0,
                                 x_offset=0, y_offset=0, astretcha=0.0, strip_len=0, max_sigma=0.08,
                                 max_disagree=0.25):
        """The correlation with the subpixel refiner where it is confident."""
        _check(self._L.xcg_correlate_device_refined(self._h, refiner._h, d_master, m_nx, m_ny, d_slave, s_nx, s_ny,
                                                    int(x_offset), int(y_offset), float(astretcha), d_locs, nlocs,
                                                    int(strip_len), d_results, float(max_sigma),
                                                    float(max_disagree), stream))

    def correlate_device(self, d_master: int, m_nx: int, m_ny: int, d_slave: int, s_nx: int, s_ny: int,
                         d_locs: int, nlocs: int, d_results: int, stream: int = 0, x_offset=0, y_offset=0,
                         astretcha=0.0, strip_len=0):
        """Device pointers in and out (integers), enqueued on `stream`."""
        _check(self._L.xcg_correlate_device(self._h, d_master, m_nx, m_ny, d_slave, s_nx, s_ny,
                                            int(x_offset), int(y_offset), float(astretcha),
                                            d_locs, nlocs, int(strip_len), d_results, stream))


class Stack:
    """A stack of pairs correlated together (xcg_stack_*).  common: ri,
    interpolation and format shared by every pair."""

    def __init__(self, common: Params, device: int = 0):
        self._L = load()
        h = ctypes.c_void_p()
        _check(self._L.xcg_stack_create(ctypes.byref(common), device, ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            self._L.xcg_stack_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _array(pairs):
        arr = (Pair * len(pairs))()
        for i, p in enumerate(pairs):
            arr[i] = p
        return arr

    def run(self, pairs, stream: int = 0):
        arr = self._array(pairs)
        _check(self._L.xcg_stack_run(self._h, arr, len(pairs), stream))

    def autotune(self, pairs, stream: int = 0):
        arr = self._array(pairs)
        _check(self._L.xcg_stack_autotune(self._h, arr, len(pairs), stream))

    def set_graph(self, on: bool):
        self._L.xcg_stack_set_graph(self._h, 1 if on else 0)

    def stats(self) -> StackStats:
        s = StackStats()
        self._L.xcg_stack_get_stats(self._h, ctypes.byref(s))
        return s


class Refiner:
    """The subpixel refiner (xcg_refiner_*): parameters, CUDA training step,
    FP32 and BF16 tensor-core forward passes."""

    def __init__(self, device: int = 0, max_batch: int = 4096):
        self._L = load()
        h = ctypes.c_void_p()
        _check(self._L.xcg_refiner_create(device, max_batch, ctypes.byref(h)))
        self._h = h
        self.max_batch = max_batch

    def close(self):
        if self._h:
            self._L.xcg_refiner_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, theta: np.ndarray):
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        assert theta.size == REFINER_NPARAM
        _check(self._L.xcg_refiner_set_params(self._h, theta.ctypes.data))

    def get_params(self) -> np.ndarray:
        out = np.zeros(REFINER_NPARAM, np.float32)
        _check(self._L.xcg_refiner_get_params(self._h, out.ctypes.data))
        return out

    def forward(self, d_feat: int, n: int, d_out: int, tensor_cores: bool = True, stream: int = 0):
        _check(self._L.xcg_refiner_forward(self._h, d_feat, n, d_out, 1 if tensor_cores else 0, stream))

    def gradient(self, d_feat: int, d_target: int, n: int, stream: int = 0):
        g = np.zeros(REFINER_NPARAM, np.float32)
        out = np.zeros((n, 3), np.float32)
        loss = ctypes.c_double()
        _check(self._L.xcg_refiner_gradient(self._h, d_feat, d_target, n, g.ctypes.data, ctypes.byref(loss),
                                            out.ctypes.data, stream))
        return loss.value, g, out

    def train_step(self, d_feat: int, d_target: int, n: int, lr: float, stream: int = 0):
        _check(self._L.xcg_refiner_train_step(self._h, d_feat, d_target, n, float(lr), stream))


def correlate_device_noalloc(p: Params, d_master: int, m_nx: int, m_ny: int, d_slave: int, s_nx: int, s_ny: int,
                             d_locs: int, nlocs: int, d_results: int, stream: int = 0, x_offset=0, y_offset=0,
                             astretcha=0.0, strip_len=0):
    """xcg_correlate_device_noalloc: device pointers in and out, no context and
    no device allocation inside the library (scratch is a fixed 32 MiB array)."""
    L = load()
    _check(L.xcg_correlate_device_noalloc(ctypes.byref(p), d_master, m_nx, m_ny, d_slave, s_nx, s_ny,
                                          int(x_offset), int(y_offset), float(astretcha), d_locs, nlocs,
                                          int(strip_len), d_results, stream))


def fit_offsets(d_results: int, d_locs: int, nlocs: int, d_out: int, ri=2, x_offset=0, y_offset=0, astretcha=0.0,
                snr_min=20.0, npar_range=3, npar_azimuth=3, robust_iters=0, stream: int = 0):
    """xcg_fit_offsets: the PRM offset model fitted on the device from a
    device result array; d_out is a device buffer of sizeof(Fit) bytes."""
    L = load()
    _check(L.xcg_fit_offsets(d_results, d_locs, int(nlocs), int(ri), int(x_offset), int(y_offset), float(astretcha),
                             float(snr_min), int(npar_range), int(npar_azimuth), int(robust_iters), d_out, stream))


def tc_gemm_check(m_tiles: int, n_tile: int, k: int, n_total: int, d_a: int, d_b: int, d_c: int, stream: int = 0):
    """xcg_tc_gemm_check: the split-FP16 tcgen05 GEMM engine on FP32 device matrices."""
    _check(load().xcg_tc_gemm_check(m_tiles, n_tile, k, n_total, d_a, d_b, d_c, stream))


def fp32_fma_rate(device: int = 0) -> float:
    """xcg_fp32_fma_rate: measured FP32 FMA throughput of the device, TFLOP/s."""
    v = ctypes.c_double()
    _check(load().xcg_fp32_fma_rate(device, ctypes.byref(v)))
    return v.value


def grid(m_nx, m_ny, nxl, nyl, xsearch=64, ysearch=64):
    """Location grid of get_locations.c:21-40 (npx = 4*xsearch, nx_corr = 2*xsearch)."""
    npx, npy = 4 * xsearch, 4 * ysearch
    x_inc = (m_nx - 2 * (xsearch + 2 * xsearch)) // (nxl + 3)
    y_inc = (m_ny - 2 * (ysearch + 2 * ysearch)) // (nyl + 1)
    return np.array([(npx + i * x_inc, npy + j * y_inc)
                     for j in range(1, nyl + 1) for i in range(2, nxl + 2)], np.int32)


def output_offsets(res, ri, x_offset, y_offset, locs_y, astretcha):
    """The offsets print_results writes (print_results.c:30-38), in float32."""
    f = np.float32
    ishft = np.trunc(np.asarray(locs_y, np.float64) * astretcha).astype(np.int32)
    xo = (res["xoff"].astype(f) / f(ri)) - (res["xfrac"].astype(f) / f(ri)) + f(x_offset)
    yo = res["yoff"].astype(f) - res["yfrac"].astype(f) + f(y_offset) + ishft.astype(f)
    return xo.astype(f), yo.astype(f)
