"""Full-size fixtures (tests/golden/c1_*): the reference's outputs for the
12 x 65,536-sample NSIDE-64 problems, with fingerprints of the inputs it saw.
The inputs themselves are regenerated with synth; a problem whose pixels do
not reproduce the stored fingerprint is skipped, not passed."""
import hashlib
import json
import math
import os

import numpy as np
import pytest

from sanepic_gb300 import synth

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FULL_NAMES = ["c1_1det_nside64", "c1_4det_nside64"]


def load_full(name):
    with open(os.path.join(GOLDEN_DIR, f"{name}_ref_log.json")) as f:
        log = json.load(f)
    z = np.load(os.path.join(GOLDEN_DIR, f"{name}_ref_outputs.npz"))
    sp = log["spec"]
    spec = synth.ProblemSpec(sp["name"], ndet=sp["ndet"], nside=sp["nside"], nseg=sp["nseg"],
                             ns=sp["ns"], hwp=sp["hwp"], fknee=sp["fknee"], alpha=sp["alpha"],
                             problem=sp["problem"], precision="f64")
    return spec, {k: z[k] for k in z.files}, log


def pixels_sha256(pix):
    return hashlib.sha256(np.ascontiguousarray(pix, np.int64).astype("<i8").tobytes()).hexdigest()


def regenerate(name, pixels_fn):
    """The problem's inputs, regenerated; skips if the RING pixels (from
    pixels_fn(prob)) or the input sums differ from those the reference saw."""
    spec, ref, log = load_full(name)
    prob = synth.make_problem(spec)
    fp = log["fingerprint"]
    for k, v in fp["sums"].items():
        got = float(np.sum(prob[k], dtype=np.float64))
        if not math.isclose(got, v, rel_tol=1e-12, abs_tol=1e-300):
            pytest.skip(f"regenerated input {k} differs from the fixture's ({got!r} vs {v!r})")
    if pixels_sha256(pixels_fn(prob)) != fp["pixels_sha256"]:
        pytest.skip("regenerated pointing gives other pixels than the fixture's")
    return spec, prob, ref, log


def map_errors(got, want, remove_monopole=False):
    """max |got - want| / max |want| and rms(got - want) / rms(want) over the
    observed pixels (want != 0); remove_monopole subtracts the mean
    difference first (the bin-0 override of sanepic.cc:536-537 leaves the
    I monopole nearly unconstrained)."""
    want = np.asarray(want, np.float64)
    obs = want != 0
    d = np.asarray(got, np.float64)[obs] - want[obs]
    if remove_monopole:
        d = d - d.mean()
    w = want[obs]
    return {"rms": float(np.sqrt(np.mean(d * d)) / np.sqrt(np.mean(w * w))),
            "max": float(np.max(np.abs(d)) / np.max(np.abs(w)))}
