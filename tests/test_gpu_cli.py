"""The drop-in xcorr program end to end on the GPU: PRM files and SLC images
on disk, the same command line as the reference, and its freq_xcorr.dat
compared with the reference's own lines (golden records).

Both ingest paths run: the default one streams bands of lines of both SLCs
while strips are correlated; XCORR_WHOLE_READ=1 reads both images whole
first.  Integer columns and offsets must match the reference's lines exactly;
the correlation column (printed %6.2f) may differ by one unit in the last
digit where the value sits on a rounding boundary."""
import os
import subprocess

import numpy as np
import pytest

import build as pkg_build
import golden_util as gu
import xcorr_gb300 as xg
from cases import CASES, PRF
from xcorr_gb300 import synth

pytestmark = pytest.mark.gpu


def _parse(lines):
    return np.array([[float(v) for v in ln.split()] for ln in lines], np.float64).reshape(-1, 5)


@pytest.fixture(scope="module")
def program():
    return pkg_build.build_cli()


@pytest.mark.parametrize("whole", [False, True], ids=["streamed", "whole"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_program_matches_reference_lines(program, tmp_path, name, whole):
    case = CASES[name]
    g = gu.load(name)
    synth.write_case(str(tmp_path), case["spec"], case.get("rshift", 0), case.get("ashift", 0), PRF,
                     case.get("prf_slave"))
    env = dict(os.environ)
    env.pop("XCORR_WHOLE_READ", None)
    if whole:
        env["XCORR_WHOLE_READ"] = "1"
    p = subprocess.run([program, "master.PRM", "aligned.PRM"] + case["flags"], cwd=tmp_path, env=env,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stderr == g["ref_stderr"]
    assert p.stdout.startswith(" elapsed time: ")
    lines = open(tmp_path / "freq_xcorr.dat").read().splitlines()
    assert len(lines) == len(g["lines"])
    a, b = _parse(lines), _parse(g["lines"])
    np.testing.assert_array_equal(a[:, [0, 2]], b[:, [0, 2]])
    np.testing.assert_array_equal(a[:, [1, 3]], b[:, [1, 3]])
    assert np.max(np.abs(a[:, 4] - b[:, 4])) <= 0.0100001
    same = sum(x == y for x, y in zip(lines, g["lines"]))
    assert same >= len(lines) - max(1, len(lines) // 200)


@pytest.mark.parametrize("flag,fname,mode", [("-time", "time_xcorr.dat", 0), ("-time4", "time_xcorr_Gatelli.dat", 1)])
def test_program_time_modes(program, tmp_path, flag, fname, mode):
    """-time / -time4 write their own file (xcorr.cu:467-469) with the lines
    the library's full-search mode gives for the same windows."""
    case = CASES["xs32"]
    g = gu.load("xs32")
    synth.write_case(str(tmp_path), case["spec"], 0, 0, PRF, None)
    p = subprocess.run([program, "master.PRM", "aligned.PRM", flag] + case["flags"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert "time cross correlation" in p.stderr
    lines = open(tmp_path / fname).read().splitlines()
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("xs32", g)
    pr = xg.params(d["xsearch"], d["ysearch"], d["ri"], d["interp_flag"], d["ifc"], corr_mode=mode)
    with xg.Context(pr) as ctx:
        r = ctx.correlate(m, s, locs, xoff, yoff, ast, strip_len=d["nxl"])
    xo_, yo_ = xg.output_offsets(r, d["ri"], xoff, yoff, locs[:, 1], ast)
    want = [" %d %6.3f %d %6.3f %6.2f " % (locs[i, 0], xo_[i], locs[i, 1], yo_[i], r["corr"][i]) for i in range(len(locs))]
    assert lines == want
