"""The drop-in `sanepic` executable: command-line and input-file handling that
ends before any GPU work (no GPU needed)."""
import os
import subprocess

import numpy as np
import pytest

from sanepic_gb300 import build, synth

CLI = build.CLI


@pytest.fixture(scope="module", autouse=True)
def _cli():
    build.build()
    assert os.path.exists(CLI)


def run(args, **kw):
    return subprocess.run([CLI] + args, capture_output=True, text=True, timeout=60, **kw)


@pytest.fixture(scope="module")
def tree(tmp_path_factory):
    spec = synth.ProblemSpec("cli", ndet=2, nside=8, nseg=2, ns=256, problem=3)
    prob = synth.make_problem(spec)
    base = str(tmp_path_factory.mktemp("tree"))
    return base, synth.write_reference_tree(prob, base)


def replace(args, flag, value):
    a = list(args)
    a[a.index(flag) + 1] = value
    return a


def test_correlated_noise_stops_like_reference(tree):
    r = run(tree[1] + ["-E", "1"])
    assert r.returncode == 0 and "NOT IMPLEMENTED YET" in r.stdout


def test_unknown_option_is_rejected(tree):
    r = run(tree[1] + ["-x", "1"])
    assert r.returncode == 1 and "not valid" in r.stderr


@pytest.mark.parametrize("flag", ["-o", "-c", "-b"])
def test_unsupported_paths_are_refused(tree, flag):
    r = run(tree[1] + [flag, "1"])
    assert r.returncode == 1 and "does not implement" in r.stderr


def test_too_few_detector_names(tree):
    args = [a for a in tree[1]]
    i = args.index("-D")
    del args[i:i + 2]
    args += ["-C", "DET0000"]
    r = run(args)
    assert r.returncode == 1 and "names" in r.stderr


def test_missing_bolometer_file(tree):
    r = run(replace(tree[1], "-X", os.path.join(tree[0], "nope.txt")))
    assert r.returncode == 1 and "offset file" in r.stderr


def test_unknown_bolometer(tree):
    base = tree[0]
    path = os.path.join(base, "bolo_info", "other.txt")
    with open(path, "w") as f:
        f.write("0 0 0.0 0.0 10.0 LFT SOMEONE\n")
    r = run(replace(tree[1], "-X", path))
    assert r.returncode == 1 and "not found" in r.stderr


def test_segment_length_mismatch(tree):
    base = tree[0]
    path = os.path.join(base, "segments", "bad.bi")
    np.array([0, 255, 256, 510], np.int64).tofile(path)
    r = run(replace(tree[1], "-f", path))
    assert r.returncode == 1 and "Problem with segment size" in r.stdout


def test_short_pointing_file(tree):
    base = tree[0]
    path = os.path.join(base, "segments", "long.bi")
    np.array([0, 255, 1 << 20, (1 << 20) + 255], np.int64).tofile(path)
    r = run(replace(tree[1], "-f", path))
    assert r.returncode == 1 and "expected" in r.stderr


def test_pol0_is_refused(tree):
    r = run(replace(tree[1], "-p", "0"))
    assert r.returncode == 1 and "pol" in r.stderr
