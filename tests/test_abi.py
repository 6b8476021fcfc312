"""C ABI checks that need no GPU: the library loads, exports every entry point
include/xcorr_gb300.h declares, and the binding's struct layouts match the
header's (compiled here with gcc)."""
import os
import re
import subprocess

import numpy as np
import pytest

import xcorr_gb300 as xg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xcorr_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xcg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = xg.load()
    names = declared_functions()
    assert names, "no declarations parsed"
    for n in names:
        assert hasattr(L, n), f"{n} declared in the header but not exported"
    assert sorted(xg.EXPORTS) == names


def test_struct_layouts_match_header(tmp_path):
    c = tmp_path / "sz.c"
    c.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "xcorr_gb300.h"\n'
                 'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(xcg_params), sizeof(xcg_loc),'
                 ' sizeof(xcg_result), offsetof(xcg_result, cmax), offsetof(xcg_result, corr0n), sizeof(xcg_stats),'
                 ' sizeof(xcg_pair), sizeof(xcg_stack_stats), sizeof(xcg_fit), offsetof(xcg_fit, azimuth));'
                 'return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I" + os.path.dirname(HEADER), str(c), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    import ctypes
    assert vals[0] == ctypes.sizeof(xg.Params)
    assert vals[1] == ctypes.sizeof(xg.Loc)
    assert vals[2] == xg.RESULT_DTYPE.itemsize
    assert vals[3] == xg.RESULT_DTYPE.fields["cmax"][1]
    assert vals[4] == xg.RESULT_DTYPE.fields["corr0n"][1]
    assert vals[5] == ctypes.sizeof(xg.Stats)
    assert vals[6] == ctypes.sizeof(xg.Pair)
    assert vals[7] == ctypes.sizeof(xg.StackStats)
    assert vals[8] == ctypes.sizeof(xg.Fit)
    assert vals[9] == xg.Fit.azimuth.offset


def test_create_rejects_bad_parameters_without_touching_the_gpu():
    # argument validation happens before any device call
    for kw in (dict(xsearch=48), dict(xsearch=8), dict(ri=3), dict(interp_factor=12), dict(corr_mode=3),
               dict(xsearch=16, corr_mode=0)):
        p = xg.params(**kw)
        with pytest.raises(xg.XcgError) as e:
            xg.Context(p)
        assert "invalid argument" in str(e.value) or "unsupported" in str(e.value)
    p = xg.params()
    p.nx_corr = 64
    with pytest.raises(xg.XcgError, match="unsupported"):
        xg.Context(p)


def test_grid_matches_get_locations():
    # get_locations.c:21-40 for a 2048 x 4096 image, nx=20, ny=50: x_inc = y_inc = 72
    g = xg.grid(2048, 4096, 20, 50)
    assert g.shape == (1000, 2)
    assert tuple(g[0]) == (256 + 2 * 72, 256 + 72)
    assert tuple(g[-1]) == (256 + 21 * 72, 256 + 50 * 72)


def test_correlate_rejects_wrong_image_layout():
    # the image checks run before the library is called (no GPU needed)
    ctx = xg.Context.__new__(xg.Context)
    ctx.params, ctx._h = xg.params(32, 32), None
    locs = np.zeros((1, 2), np.int32)
    with pytest.raises(ValueError):
        ctx.correlate(np.zeros((8, 8), np.float32), np.zeros((8, 8), np.float32), locs)
    with pytest.raises(ValueError):
        ctx.correlate(np.zeros((8, 8, 2), np.int32), np.zeros((8, 8, 2), np.int16), locs)
    ctx.params = xg.params(32, 32, fmt=1)
    with pytest.raises(ValueError):
        ctx.correlate(np.zeros((8, 8, 2), np.int16), np.zeros((8, 8, 2), np.int16), locs)
