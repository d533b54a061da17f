"""Runs the reference's gain recalibration (-r, sanepic.cc:2108-2316) as
built against the project's shims (oracle/_ref/sanepic) on a small problem
with known gain errors, and prints its recalibration lines.

The problem: the 4-detector NSIDE-16 golden inputs (tests/golden) with every
(detector, segment) timeline multiplied by a gain 1 + 0.02 N(0, 1), and
all-zero orbital-dipole timelines (the reference reads orbdip_<detector>
whenever -r is set, sanepic.cc:702-712).  Usage, where the reference was
built (make -C oracle ref REFERENCE_SRC=<checkout>/src/sanepic.cc):

    python oracle/probe_recalib.py            # -r 1
    python oracle/probe_recalib.py --global   # -r 1 -R 1
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from golden_util import load_problem  # noqa: E402
from sanepic_gb300 import synth  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--global", dest="glob", action="store_true", help="also -R 1")
    a = ap.parse_args()
    prob = load_problem("golden_4det_nside16")
    spec = prob["spec"]
    g = 1.0 + 0.02 * np.random.default_rng(1).standard_normal((spec.ndet, spec.nseg))
    tod = prob["tod"].copy()
    for d in range(spec.ndet):
        for s in range(spec.nseg):
            tod[d, s * spec.ns:(s + 1) * spec.ns] *= g[d, s]
    prob["tod"] = tod
    with tempfile.TemporaryDirectory() as td:
        args = synth.write_reference_tree(prob, td)
        for name in prob["names"]:
            np.zeros(spec.nseg * spec.ns).tofile(os.path.join(td, "tod_list", f"orbdip_{name}"))
        args += ["-r", "1"] + (["-R", "1"] if a.glob else [])
        r = subprocess.run(["stdbuf", "-oL", os.path.join(HERE, "_ref", "sanepic")] + args,
                           env=dict(os.environ, SHIM_MPI_NP="3"), capture_output=True,
                           text=True, timeout=1200, cwd=td)
    print("rc", r.returncode)
    for line in r.stdout.splitlines():
        if re.match(r"(Before|After) recal|recal =|var0 =", line):
            print(line)


if __name__ == "__main__":
    main()
