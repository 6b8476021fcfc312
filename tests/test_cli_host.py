"""The drop-in program's host side against the reference's own host C code.

oracle/_ref/ref_host_probe runs the reference's set_defaults /
parse_command_line / handle_prm / get_locations / print_results
(parse_xcorr_input.c, sio_struct.c, get_locations.c, print_results.c) on a
command line; `xcorr` with XCORR_DRY_RUN=1 prints the same things from its own
code.  Both must agree byte for byte.  No GPU is used."""
import os
import subprocess

import numpy as np
import pytest

from xcorr_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_host_probe")
CLI = os.path.join(ROOT, "gmtsar-gpu_gb300", "bin", "xcorr")

needs_probe = pytest.mark.skipif(not os.path.exists(PROBE), reason="reference host probe not built (no reference sources)")


@pytest.fixture(scope="module")
def cli():
    import build as pkg_build
    pkg_build.build_all()
    return CLI


def _prms(d, m_nx=2048, m_ny=4096, s_nx=2048, s_ny=4096, rshift=0, ashift=0, prf2=1679.9):
    for name, nx, ny in (("master.SLC", m_nx, m_ny), ("aligned.SLC", s_nx, s_ny)):
        open(os.path.join(d, name), "wb").close()
    synth.write_prm(os.path.join(d, "master.PRM"), "master.SLC", m_nx, m_ny, 0, 0, 1679.9)
    synth.write_prm(os.path.join(d, "aligned.PRM"), "aligned.SLC", s_nx, s_ny, rshift, ashift, prf2)


def _run(exe, d, flags, env_extra):
    env = dict(os.environ, **env_extra)
    p = subprocess.run([exe, "master.PRM", "aligned.PRM"] + flags, cwd=d, env=env, capture_output=True, text=True)
    return p


COMMANDS = [
    (dict(), ["-nx", "20", "-ny", "50"]),
    (dict(), []),
    (dict(m_nx=10240, m_ny=30720, s_nx=10240, s_ny=30720), ["-nx", "100", "-ny", "400", "-xsearch", "128", "-ysearch", "128"]),
    (dict(rshift=5, ashift=-7, prf2=1679.9 * 1.002), ["-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "32"]),
    (dict(rshift=5, ashift=-7, prf2=1679.9 * 1.002), ["-noshift", "-nx", "7", "-ny", "3"]),
    (dict(), ["-norange", "-interp", "8", "-xsearch", "32", "-ysearch", "64", "-nx", "5", "-ny", "9"]),
    (dict(), ["-range_interp", "4", "-nointerp", "-real", "-v"]),
]


@needs_probe
@pytest.mark.parametrize("prm,flags", COMMANDS)
def test_parameters_and_grid_match_reference(tmp_path, cli, prm, flags):
    _prms(str(tmp_path), **prm)
    ref = _run(PROBE, str(tmp_path), flags, {})
    ours = _run(cli, str(tmp_path), flags, {"XCORR_DRY_RUN": "1"})
    assert ref.returncode == 0, ref.stderr
    assert ours.returncode == 0, ours.stderr
    assert ours.stdout == ref.stdout
    # the progress lines on stderr match too
    want = [l for l in ref.stderr.splitlines() if l.strip()]
    got = [l for l in ours.stderr.splitlines() if l.strip()]
    assert got == want


@needs_probe
def test_result_lines_match_print_results(tmp_path, cli):
    _prms(str(tmp_path), rshift=3, ashift=-2, prf2=1679.9 * 1.0005)
    rng = np.random.default_rng(4)
    rows = []
    for i in range(400):
        x, y = int(rng.integers(0, 5000)), int(rng.integers(0, 30000))
        xoff, yoff = float(rng.integers(-64, 64)), float(rng.integers(-64, 64))
        xfrac, yfrac = rng.integers(-64, 64) / 16.0, rng.integers(-64, 64) / 16.0
        corr = float(np.float32(rng.uniform(0, 100)))
        if i % 7 == 0:
            xoff, xfrac, yoff, yfrac = -0.0, 0.0, -0.0, 0.0
        rows.append(f"{x} {y} {xoff!r} {yoff!r} {xfrac!r} {yfrac!r} {corr!r}")
    f = tmp_path / "vals.txt"
    f.write_text("\n".join(rows) + "\n")
    for flags in ([], ["-norange"], ["-range_interp", "4"]):
        ref = _run(PROBE, str(tmp_path), flags, {"XCG_PROBE_PRINT": str(f)})
        ours = _run(cli, str(tmp_path), flags, {"XCORR_DRY_RUN": "1", "XCORR_PRINT_FILE": str(f)})
        assert ref.returncode == 0 and ours.returncode == 0
        assert ours.stdout == ref.stdout


def test_unknown_option_and_bad_search_are_rejected(tmp_path, cli):
    _prms(str(tmp_path))
    p = _run(cli, str(tmp_path), ["-bogus"], {"XCORR_DRY_RUN": "1"})
    assert p.returncode == 1 and "option not recognized" in p.stderr
    p = _run(cli, str(tmp_path), ["-xsearch", "48"], {"XCORR_DRY_RUN": "1"})
    assert p.returncode == 1 and "power of 2" in p.stderr
    p = _run(cli, str(tmp_path), ["-nx"], {"XCORR_DRY_RUN": "1"})
    assert p.returncode == 1 and "no option after -nx" in p.stderr


def test_missing_files_are_reported(tmp_path, cli):
    p = _run(cli, str(tmp_path), [], {"XCORR_DRY_RUN": "1"})
    assert p.returncode == 1 and "Can't open prmfile" in p.stderr
    synth.write_prm(str(tmp_path / "master.PRM"), "nothere.SLC", 100, 100)
    synth.write_prm(str(tmp_path / "aligned.PRM"), "nothere.SLC", 100, 100)
    p = _run(cli, str(tmp_path), [], {"XCORR_DRY_RUN": "1"})
    assert p.returncode == 1 and "Cannot open SLC_file" in p.stderr


def test_integration_doc_shows_the_built_shim():
    """INTEGRATION.md section 2 shows the shim that oracle/ref/build_ref.sh
    builds and tests/test_gpu_shim.py runs, character for character."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    doc = open(os.path.join(root, "INTEGRATION.md")).read()
    shim = open(os.path.join(root, "gmtsar-gpu_gb300", "integration", "do_correlation_shim.cpp")).read()
    assert "```cpp\n" + shim + "```" in doc
