"""Generate the gain-recalibration fixture from the reference itself.

Runs the UNMODIFIED reference (patanch/SANEPIC src/sanepic.cc, built by
`make -C oracle ref` against the project-written FFTW/MPI shims) with -r 1
and with -r 1 -R 1 on golden problems (the 4-detector NSIDE-16 one, and the
2-detector one with a half-wave plate) whose (detector, segment) timelines
were multiplied by gains 1 + 0.02 N(0, 1) (numpy default_rng(1), shape
[ndet][nseg]), with all-zero orbital-dipole timelines (the reference reads
orbdip_<detector> whenever -r is set, sanepic.cc:702-712), and stores what
its first gain fit prints before its loop diverges:

  recal_<tag>_ref.npz   A_1: the compact map of its first loop
                        (map_A_..._1, made with gains 1), and the gains
                        applied to the timelines
  recal_<tag>_ref.json  per run: the first "Before recal chi2", "After
                        recal chi2" and (-R) the ndet "Coef calib det" lines

Usage (needs the reference checkout, this container only):
    python tests/golden/make_recal_golden.py --ref-src <checkout>/src/sanepic.cc
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from golden_util import load_problem  # noqa: E402
from sanepic_gb300 import synth  # noqa: E402

# fixture tag -> golden problem
PROBLEMS = {"4det_nside16": "golden_4det_nside16",
            "2det_nside16_hwp": "golden_2det_nside16_hwp"}
NPROC = 3  # 1 master + 2 workers, as the other golden runs


def recal_problem(name="golden_4det_nside16"):
    """The golden problem with its timelines times the seeded gains."""
    prob = load_problem(name)
    spec = prob["spec"]
    g = 1.0 + 0.02 * np.random.default_rng(1).standard_normal((spec.ndet, spec.nseg))
    tod = prob["tod"].copy()
    for d in range(spec.ndet):
        for s in range(spec.nseg):
            tod[d, s * spec.ns:(s + 1) * spec.ns] *= g[d, s]
    prob["tod"] = tod
    return prob, g


def run(prob, exe, extra):
    spec = prob["spec"]
    with tempfile.TemporaryDirectory() as td:
        args = synth.write_reference_tree(prob, td)
        for name in prob["names"]:
            np.zeros(spec.nseg * spec.ns).tofile(os.path.join(td, "tod_list", f"orbdip_{name}"))
        r = subprocess.run(["stdbuf", "-oL", exe] + args + extra,
                           env=dict(os.environ, SHIM_MPI_NP=str(NPROC)), capture_output=True,
                           text=True, timeout=1800, cwd=td)
        names = synth.output_names(spec, os.path.join(td, "out_dir", "map_"))
        a1 = np.fromfile(names["A"], dtype="<f8")
    if r.returncode != 0:
        raise RuntimeError(f"reference failed rc={r.returncode}\n{r.stdout[-2000:]}")
    out = {"before": None, "after": None, "coef": []}
    for line in r.stdout.splitlines():
        m = re.match(r"Before recal chi2 = (\S+)", line)
        if m and out["before"] is None:
            out["before"] = float(m.group(1))
        m = re.match(r"After recal chi2 = (\S+)", line)
        if m and out["after"] is None:
            out["after"] = float(m.group(1))
        m = re.match(r"Coef calib det (\d+) is (\S+)", line)
        if m and len(out["coef"]) < spec.ndet:
            out["coef"].append(float(m.group(2)))
    return a1, out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True, help="the reference's src/sanepic.cc")
    a = ap.parse_args()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref",
                           f"REFERENCE_SRC={a.ref_src}"])
    exe = os.path.join(ROOT, "oracle", "_ref", "sanepic")
    for tag, name in PROBLEMS.items():
        prob, g = recal_problem(name)
        a_tile, tile = run(prob, exe, ["-r", "1"])
        a_det, det = run(prob, exe, ["-r", "1", "-R", "1"])
        if not np.array_equal(a_tile, a_det):
            raise RuntimeError("the first loop's map differs between the two runs")
        np.savez_compressed(os.path.join(HERE, f"recal_{tag}_ref.npz"), A_1=a_tile, gains=g)
        with open(os.path.join(HERE, f"recal_{tag}_ref.json"), "w") as f:
            json.dump({"problem": name, "gain_seed": 1, "gain_sigma": 0.02, "nproc": NPROC,
                       "per_tile": tile, "per_detector": det,
                       "generator": "tests/golden/make_recal_golden.py"}, f, indent=1)
        print(tag, "per tile", tile)
        print(tag, "per detector", det)


if __name__ == "__main__":
    main()
