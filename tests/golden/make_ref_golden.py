"""Run the reference xcorr-gpu on the golden cases and record its output.

Needs a GPU and the reference program built by oracle/ref/build_ref.sh
(oracle/_ref/xcorr-gpu-dump).  For each case in cases.py it writes the
synthetic SLC pair and PRM files into a scratch directory, runs the reference
there, and stores ref_<case>.json.gz in --out with: the generator spec, the
command line, SHA-256 of both images, every freq_xcorr.dat line, and the
full-precision per-location dump (struct locs fields plus the reduction
results cmax, cave, ip, jp, the fine peak and both patch means).

usage: python tests/golden/make_ref_golden.py --out DIR [--cases a,b] [--work DIR]
"""
import argparse
import gzip
import json
import os
import shutil
import subprocess
import sys
import time

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, _HERE)
from cases import CASES, PRF  # noqa: E402
from xcorr_gb300 import synth  # noqa: E402

REF_BIN = os.path.join(_HERE, "..", "..", "oracle", "_ref", "xcorr-gpu-dump")
DUMP_COLS = ["iloc", "x", "y", "xoff", "yoff", "xfrac", "yfrac", "corr", "cmax", "cave",
             "ip", "jp", "fip", "fjp", "fmax", "mean1", "mean2"]


def run_case(name, case, work, out):
    d = os.path.join(work, name)
    shutil.rmtree(d, ignore_errors=True)
    spec = case["spec"]
    m, s = synth.write_case(d, spec, case.get("rshift", 0), case.get("ashift", 0), PRF,
                            case.get("prf_slave"))
    cmd = [os.path.abspath(REF_BIN), "master.PRM", "aligned.PRM"] + case["flags"]
    env = dict(os.environ, XCG_REF_DUMP=os.path.join(d, "ref_dump.txt"))
    t0 = time.time()
    p = subprocess.run(cmd, cwd=d, env=env, capture_output=True, text=True, timeout=900)
    wall = time.time() - t0
    if p.returncode != 0:
        raise SystemExit(f"{name}: reference exited {p.returncode}\n{p.stdout[-2000:]}\n{p.stderr[-2000:]}")
    lines = open(os.path.join(d, "freq_xcorr.dat")).read().splitlines()
    dump = []
    for ln in open(os.path.join(d, "ref_dump.txt")):
        if ln.startswith("#"):
            continue
        v = ln.split()
        row = [float(x) if ("." in x or "e" in x or "n" in x.lower()) else int(x) for x in v]
        dump.append(row)
    rec = dict(case=name, spec=spec.to_dict(), flags=case["flags"],
               rshift=case.get("rshift", 0), ashift=case.get("ashift", 0), prf_master=PRF,
               prf_slave=case.get("prf_slave", PRF),
               sha256=dict(master=synth.sha256(m), slave=synth.sha256(s)),
               lines=lines, dump_cols=DUMP_COLS, dump=dump, ref_wall_s=wall,
               ref_stdout=p.stdout[-4000:], ref_stderr=p.stderr[-4000:])
    os.makedirs(out, exist_ok=True)
    with gzip.open(os.path.join(out, f"ref_{name}.json.gz"), "wt") as f:
        json.dump(rec, f)
    print(f"{name}: {len(lines)} locations, reference wall {wall:.2f} s", flush=True)
    shutil.rmtree(d, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--work", default="/tmp/xcg_golden_work")
    ap.add_argument("--cases", default=",".join(CASES))
    a = ap.parse_args()
    for name in a.cases.split(","):
        run_case(name, CASES[name], a.work, a.out)


if __name__ == "__main__":
    main()
