"""Generate the golden fixtures in this directory from the reference itself.

Runs the UNMODIFIED reference (patanch/SANEPIC src/sanepic.cc, built by
`make -C oracle ref` against the project-written FFTW/MPI shims) on small
seeded synthetic problems and stores, per problem:

  <name>_inputs.npz      the exact inputs (pointing, detectors, iSpf, TOD)
  <name>_ref_outputs.npz every map the reference writes (full RING, FP64)
  <name>_ref_log.json    its "iter = .., crit = .." sequence and run metadata

The inputs are stored (not regenerated) so the fixtures do not depend on the
host's libm.  Usage (needs the reference checkout, this container only):
    python tests/golden/make_golden.py --ref-src <reference checkout>/src/sanepic.cc
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

from sanepic_gb300 import synth  # noqa: E402

GOLDEN = {
    # 4 detectors, NSIDE 16, 16 x 2048 samples, 1/f noise, no HWP
    "golden_4det_nside16": synth.ProblemSpec(
        "golden_4det_nside16", ndet=4, nside=16, nseg=16, ns=2048, fknee=0.02,
        alpha=1.0, problem=0),
    # 2 detectors, NSIDE 16, 8 x 4096 samples, HWP on
    "golden_2det_nside16_hwp": synth.ProblemSpec(
        "golden_2det_nside16_hwp", ndet=2, nside=16, nseg=8, ns=4096, fknee=0.1,
        alpha=1.0, hwp=True, problem=1),
}
NPROC = 3  # 1 master + 2 workers (the reference needs >= 2 ranks)

# Full-size problems (12 x 65,536 samples per detector, NSIDE 64): too large
# to store their inputs, so only the reference's outputs, its iteration log and
# fingerprints of the inputs are stored; tests regenerate the inputs with
# synth and skip when the fingerprints differ.
FULL_SIZE = {
    # the 1-detector workload (1 det, NSIDE 64, 12 x 65,536, 1/f fknee 0.1 Hz):
    # one detector angle leaves most Q/U blocks nearly singular, and the
    # reference stops at its 2000-iteration limit without converging
    "c1_1det_nside64": synth.spec_from_name("c1_1det_nside64"),
    # the same scan and sizes with 4 detectors at seeded orientations: well
    # posed, the reference converges to its own 1e-15 stop
    "c1_4det_nside64": synth.ProblemSpec(
        "c1_4det_nside64", ndet=4, nside=64, nseg=12, ns=65536, fknee=0.1, alpha=1.0,
        problem=3),
}
NPROC_FULL = 5  # 1 master + 4 workers


def save_inputs(prob, path):
    np.savez_compressed(
        path, ra=prob["ra"], dec=prob["dec"], psi=prob["psi"],
        isampmin=prob["isampmin"], angles=prob["angles"], omega=prob["omega"],
        ispf=prob["ispf"], tod=prob["tod"], names=np.array(prob["names"]),
        dims=np.array([prob["spec"].ndet, prob["spec"].nside, prob["spec"].nseg,
                       prob["spec"].ns, int(prob["spec"].hwp)], np.int64))


def fingerprint(prob):
    """Fingerprints of a problem's inputs: SHA-256 of the RING pixel of every
    sample (computed by the oracle, which reproduces the reference's
    datatopix bit for bit) and of the raw FP64 input bytes, plus sums that
    tolerate last-bit differences of the host's libm."""
    import hashlib

    import oracle
    s = oracle.Setup(prob)
    raw = hashlib.sha256()
    for k in ("ra", "dec", "psi", "ispf", "tod"):
        raw.update(np.ascontiguousarray(prob[k], np.float64).tobytes())
    return {"pixels_sha256": hashlib.sha256(s.pix.astype("<i8").tobytes()).hexdigest(),
            "inputs_sha256": raw.hexdigest(),
            "sums": {k: float(np.sum(prob[k], dtype=np.float64))
                     for k in ("ra", "dec", "psi", "ispf", "tod")},
            "npix": int(s.npix)}


def run_reference(prob, exe, workdir, nproc=NPROC):
    args = synth.write_reference_tree(prob, workdir)
    env = dict(os.environ, SHIM_MPI_NP=str(nproc))
    r = subprocess.run(["stdbuf", "-oL", exe] + args, env=env, capture_output=True,
                       text=True, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed rc={r.returncode}\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    crit = []
    for line in r.stdout.splitlines():
        m = re.match(r"iter = (\d+), crit = (\S+), crit2 = (\S+), chi2 = (\S+)", line)
        if m:
            crit.append([int(m.group(1)), float(m.group(2)), float(m.group(3)),
                         float(m.group(4))])
    names = synth.output_names(prob["spec"], os.path.join(workdir, "out_dir", "map_"))
    outs = {k: np.fromfile(v, dtype="<f8") for k, v in names.items()}
    return outs, crit, r.stdout


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True, help="the reference's src/sanepic.cc")
    ap.add_argument("--full-size", action="store_true",
                    help="only the full-size problems (outputs and fingerprints)")
    a = ap.parse_args()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref",
                           f"REFERENCE_SRC={a.ref_src}"])
    exe = os.path.join(ROOT, "oracle", "_ref", "sanepic")
    if a.full_size:
        import time
        for name, spec in FULL_SIZE.items():
            prob = synth.make_problem(spec)
            with tempfile.TemporaryDirectory() as td:
                t = time.time()
                outs, crit, _ = run_reference(prob, exe, td, NPROC_FULL)
                wall = time.time() - t
            keep = ("I", "Q", "U", "NVAR", "HITS", "POL_HITS", "COS2P", "SIN2P")
            np.savez_compressed(os.path.join(HERE, f"{name}_ref_outputs.npz"),
                                **{k: outs[k] for k in keep})
            with open(os.path.join(HERE, f"{name}_ref_log.json"), "w") as f:
                json.dump({"spec": {k: getattr(spec, k) for k in
                                    ("name", "ndet", "nside", "nseg", "ns", "hwp", "fknee",
                                     "alpha", "problem")},
                           "nproc": NPROC_FULL, "iterations": len(crit), "crit": crit,
                           "fingerprint": fingerprint(prob), "wall_seconds": wall,
                           "generator": "tests/golden/make_golden.py --full-size"}, f)
            print(name, "iterations", len(crit), "final crit", crit[-1][1], "wall", wall)
        return
    for name, spec in GOLDEN.items():
        prob = synth.make_problem(spec)
        with tempfile.TemporaryDirectory() as td:
            outs, crit, stdout = run_reference(prob, exe, td)
        save_inputs(prob, os.path.join(HERE, f"{name}_inputs.npz"))
        np.savez_compressed(os.path.join(HERE, f"{name}_ref_outputs.npz"), **outs)
        with open(os.path.join(HERE, f"{name}_ref_log.json"), "w") as f:
            json.dump({"spec": {k: getattr(spec, k) for k in
                                ("ndet", "nside", "nseg", "ns", "hwp", "fknee", "alpha",
                                 "problem")},
                       "nproc": NPROC, "iterations": len(crit), "crit": crit,
                       "generator": "tests/golden/make_golden.py"}, f, indent=1)
        print(name, "iterations", len(crit), "final crit", crit[-1][1] if crit else None)


if __name__ == "__main__":
    main()
