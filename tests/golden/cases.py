"""Golden cases: synthetic SLC pairs + xcorr command lines.

Each case is run through the reference program (built from the reference
sources by oracle/ref/build_ref.sh) by make_ref_golden.py; its per-location
output is committed as ref_<name>.json.gz.  The tests regenerate the same
inputs from the seeds below and check the oracle and the GPU path against
those files.  Every case keeps nxl a multiple of 4: the reference's transpose
kernel places a barrier inside a bounds branch (fft_interpolate_routines.cu:27-40)
and is not run on partial tiles.
"""
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(_HERE, "..", "..", "gmtsar-gpu_gb300", "python"))
from xcorr_gb300.synth import PairSpec  # noqa: E402

PRF = 1679.9

CASES = {
    # 1000 windows of 128^2 (256^2 FFT), the headline configuration
    "cfg1": dict(spec=PairSpec(nx=2048, ny=4096, dx=3.37, dy=-5.81, noise_frac=0.1, seed=11),
                 flags=["-nx", "20", "-ny", "50"]),
    "xs32": dict(spec=PairSpec(nx=1024, ny=1536, dx=-2.3, dy=1.6, noise_frac=0.2, seed=12),
                 flags=["-nx", "8", "-ny", "12", "-xsearch", "32", "-ysearch", "32"]),
    "aniso": dict(spec=PairSpec(nx=1024, ny=2048, dx=1.2, dy=-7.45, noise_frac=0.3, seed=13),
                  flags=["-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "64"]),
    "norange_i8": dict(spec=PairSpec(nx=1024, ny=1536, dx=0.71, dy=2.2, noise_frac=0.1, seed=14),
                       flags=["-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "32", "-norange", "-interp", "8"]),
    "ri4_i32": dict(spec=PairSpec(nx=1024, ny=1536, dx=-3.1, dy=-0.8, noise_frac=0.1, seed=18),
                    flags=["-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "32", "-range_interp", "4",
                           "-interp", "32"]),
    "prmshift": dict(spec=PairSpec(nx=1536, ny=2048, dx=5.4, dy=-7.3, noise_frac=0.1, seed=15),
                     rshift=5, ashift=-7, prf_slave=PRF * (1 + 2e-3),
                     flags=["-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "32"]),
    "noshift": dict(spec=PairSpec(nx=1536, ny=2048, dx=5.4, dy=-7.3, noise_frac=0.1, seed=15),
                    rshift=5, ashift=-7, prf_slave=PRF * (1 + 2e-3),
                    flags=["-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "32", "-noshift"]),
    "real": dict(spec=PairSpec(nx=1024, ny=1536, dx=-1.37, dy=0.45, noise_frac=0.1, seed=16, real=True),
                 flags=["-real", "-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "32"]),
    # rows 340..509 of the master are zero: strip 2 sees all-zero master patches
    # (zero surface, gamma denominator 0, NaN normalisation), strip 1 a partial band
    "zeroband": dict(spec=PairSpec(nx=1024, ny=1536, dx=2.0, dy=-1.5, noise_frac=0.1, seed=17, zero_rows=(340, 510)),
                     flags=["-nx", "8", "-ny", "8", "-xsearch", "32", "-ysearch", "32"]),
}
