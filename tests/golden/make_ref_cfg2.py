"""Run the reference xcorr-gpu on the full-frame configuration and record
its per-location results compactly.

Full frame: 10240 (range) x 30720 (azimuth) complex-int16 speckle pair, a
spatially varying shift dx = 2.1 + 1e-5 x - 3e-6 y, dy = -4.7 + 2e-6 x + 8e-6 y
(xcorr_gb300.synth.make_pair_varying, piecewise constant over 512-px
blocks), 20 dB SNR; 100 x 400 = 40000 locations, xsearch = ysearch = 128.
Needs a GPU (the generator uses torch.fft on it) and the reference program
built by oracle/ref/build_ref.sh.  Writes --out/ref_cfg2.npz with the integer
and fine peaks, corr, cmax and the SHA-256 of both images, and prints the
reference's wall time.

usage: python tests/golden/make_ref_cfg2.py --out DIR [--work DIR]
"""
import argparse
import os
import shutil
import subprocess
import sys
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(_HERE, "..", "..", "gmtsar-gpu_gb300", "python"))
from xcorr_gb300 import synth  # noqa: E402

REF_BIN = os.path.join(_HERE, "..", "..", "oracle", "_ref", "xcorr-gpu-dump")
NX, NY = 10240, 30720
FLAGS = ["-nx", "100", "-ny", "400", "-xsearch", "128", "-ysearch", "128"]
NOISE = 0.01          # 20 dB
SEED = 2


def make_inputs():
    return synth.make_pair_varying(NX, NY, synth.cfg2_shift, NOISE, seed=SEED)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--work", default="/tmp/xcg_cfg2_work")
    a = ap.parse_args()
    shutil.rmtree(a.work, ignore_errors=True)
    os.makedirs(a.work)
    t0 = time.time()
    m, s, _ = make_inputs()
    m.tofile(os.path.join(a.work, "master.SLC"))
    s.tofile(os.path.join(a.work, "aligned.SLC"))
    synth.write_prm(os.path.join(a.work, "master.PRM"), "master.SLC", NX, NY)
    synth.write_prm(os.path.join(a.work, "aligned.PRM"), "aligned.SLC", NX, NY)
    print(f"inputs {time.time() - t0:.1f} s", flush=True)
    env = dict(os.environ, XCG_REF_DUMP=os.path.join(a.work, "ref_dump.txt"))
    t0 = time.time()
    p = subprocess.run([os.path.abspath(REF_BIN), "master.PRM", "aligned.PRM"] + FLAGS, cwd=a.work, env=env,
                       capture_output=True, text=True, timeout=3000)
    wall = time.time() - t0
    if p.returncode != 0:
        raise SystemExit(f"reference exited {p.returncode}: {p.stderr[-2000:]}")
    rows = [ln.split() for ln in open(os.path.join(a.work, "ref_dump.txt")) if not ln.startswith("#")]
    D = np.array([[float(v) for v in r] for r in rows])
    os.makedirs(a.out, exist_ok=True)
    np.savez_compressed(os.path.join(a.out, "ref_cfg2.npz"),
                        x=D[:, 1].astype(np.int32), y=D[:, 2].astype(np.int32),
                        ip=D[:, 10].astype(np.int16), jp=D[:, 11].astype(np.int16),
                        fip=D[:, 12].astype(np.int16), fjp=D[:, 13].astype(np.int16),
                        corr=D[:, 7].astype(np.float32), cmax=D[:, 8], cave=D[:, 9],
                        sha_master=np.array(synth.sha256(m)), sha_slave=np.array(synth.sha256(s)),
                        ref_wall_s=np.array(wall), ref_stdout=np.array(p.stdout[-2000:]))
    print(f"reference: {len(rows)} locations in {wall:.1f} s wall", flush=True)
    shutil.rmtree(a.work, ignore_errors=True)


if __name__ == "__main__":
    main()
