"""The reference-side binding of INTEGRATION.md built and run: the reference
program with its own main, option parser, PRM reader, location grid and
result writer, its do_correlation replaced by the library call of
gmtsar-gpu_gb300/integration/do_correlation_shim.cpp (linked by
oracle/ref/build_ref.sh as oracle/_ref/xcorr-gb300-shim).

The program is built only where the reference sources are at hand
(XCG_REFERENCE_SOURCES at build time); elsewhere these tests skip.  Its
freq_xcorr.dat must equal the drop-in program's and match the reference's
own lines as tests/test_gpu_cli.py requires of the drop-in program."""
import os
import subprocess

import numpy as np
import pytest

import build as pkg_build
import golden_util as gu
from cases import CASES, PRF
from xcorr_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "oracle", "_ref", "xcorr-gb300-shim")


def _parse(lines):
    return np.array([[float(v) for v in ln.split()] for ln in lines], np.float64).reshape(-1, 5)


@pytest.mark.skipif(not os.access(SHIM, os.X_OK), reason="the reference program with the shim is built only where "
                                                        "its sources are (XCG_REFERENCE_SOURCES)")
@pytest.mark.parametrize("name", ["cfg1", "xs32", "prmshift", "real", "zeroband"])
def test_reference_program_with_library_call(tmp_path, name):
    case = CASES[name]
    g = gu.load(name)
    synth.write_case(str(tmp_path), case["spec"], case.get("rshift", 0), case.get("ashift", 0), PRF,
                     case.get("prf_slave"))
    p = subprocess.run([SHIM, "master.PRM", "aligned.PRM"] + case["flags"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert "with libxcorr_gb300" in p.stderr          # the shim's do_correlation ran, not the reference's
    assert p.stdout.startswith(" elapsed time: ")     # the reference's own main
    shim_lines = open(tmp_path / "freq_xcorr.dat").read().splitlines()
    os.remove(tmp_path / "freq_xcorr.dat")
    q = subprocess.run([pkg_build.build_cli(), "master.PRM", "aligned.PRM"] + case["flags"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert q.returncode == 0, q.stderr[-2000:]
    assert shim_lines == open(tmp_path / "freq_xcorr.dat").read().splitlines()
    a, b = _parse(shim_lines), _parse(g["lines"])
    np.testing.assert_array_equal(a[:, :4], b[:, :4])
    assert np.max(np.abs(a[:, 4] - b[:, 4])) <= 0.0100001
