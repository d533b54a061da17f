"""The drop-in `sanepic` executable on the reference's own file tree: same
command line, same output files, same printed iteration lines (golden
fixtures made by the unmodified reference)."""
import os
import re
import subprocess

import numpy as np
import pytest

from golden_util import NAMES, load_log, load_outputs, load_problem, rel_rms
from sanepic_gb300 import build, synth

pytestmark = pytest.mark.gpu

ITER = re.compile(r"iter = (\d+), crit = (\S+), crit2 = (\S+), chi2 = (\S+)")


@pytest.fixture(scope="module", autouse=True)
def _cli():
    build.build()


def read_map(path):
    return np.fromfile(path, dtype="<f8")


@pytest.mark.parametrize("name", NAMES)
def test_cli_outputs_match_reference(name, tmp_path):
    prob = load_problem(name)
    ref = load_outputs(name)
    log = load_log(name)
    args = synth.write_reference_tree(prob, str(tmp_path))
    args[args.index("-i") + 1] = "1"  # also write the running maps every -j iterations
    args += ["-j", "10"]
    env = dict(os.environ, SANEPIC_GPU_PRECOND="diag", SANEPIC_GPU_PRECISION="f64")
    r = subprocess.run([build.CLI] + args, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = np.array([[float(v) for v in m.groups()] for m in ITER.finditer(r.stdout)])
    ref_rows = np.array(log["crit"])
    assert len(rows) > 10
    n = min(10, len(ref_rows))
    np.testing.assert_allclose(rows[:n, 1], ref_rows[:n, 1], rtol=1e-6)  # crit
    np.testing.assert_allclose(rows[:n, 2], ref_rows[:n, 2], rtol=1e-6)  # crit2
    np.testing.assert_allclose(rows[:n, 3], ref_rows[:n, 3], rtol=1e-9)  # chi2
    assert abs(len(rows) - log["iterations"]) <= max(3, log["iterations"] // 10)

    spec = prob["spec"]
    names = synth.output_names(spec, os.path.join(str(tmp_path), "out_dir", "map_"))
    npixfull = 12 * spec.nside ** 2
    for k in ("HITS", "POL_HITS"):
        assert np.array_equal(read_map(names[k]), ref[k]), k
    for k in ("COS2P", "SIN2P", "NVAR", "Q_NVAR", "U_NVAR"):
        m = read_map(names[k])
        assert m.size == npixfull
        assert rel_rms(m, ref[k]) < 1e-10, k
    assert rel_rms(read_map(names["I"]), ref["I"], remove_monopole=True) < 1e-6
    assert rel_rms(read_map(names["Q"]), ref["Q"]) < 1e-6
    assert rel_rms(read_map(names["U"]), ref["U"]) < 1e-6
    a = read_map(names["A"])
    npix = int((ref["HITS"] > 0).sum())
    assert a.size == 3 * npix
    e = f"output_N{spec.nside}_.bin"
    out = os.path.join(str(tmp_path), "out_dir", "map_")
    for it in (0, 10):
        for c in "IQU":
            assert read_map(f"{out}_{c}{e}_{it}").size == npixfull


def test_cli_restart_from_its_own_start_map(tmp_path):
    # -I: a run stopped early writes its compact solution (map__A_*,
    # sanepic.cc:1786-1788); a second run started from it (sanepic.cc:
    # 1209-1227) converges to the maps of one uninterrupted run
    name = NAMES[0]
    prob = load_problem(name)
    spec = prob["spec"]
    runs = {}
    for tag, stop, init in (("full", "1e-15", None), ("first", "1e-6", None),
                            ("resumed", "1e-15", "first")):
        d = tmp_path / tag
        d.mkdir()
        args = synth.write_reference_tree(prob, str(d))
        if init:
            args += ["-I", runs[init]["names"]["A"]]
        env = dict(os.environ, SANEPIC_GPU_PRECOND="diag", SANEPIC_GPU_PRECISION="f64",
                   SANEPIC_GPU_STOP=stop)
        r = subprocess.run([build.CLI] + args, capture_output=True, text=True, timeout=600,
                           env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        rows = np.array([[float(v) for v in m.groups()] for m in ITER.finditer(r.stdout)])
        runs[tag] = {"rows": rows,
                     "names": synth.output_names(spec, os.path.join(str(d), "out_dir", "map_"))}
    first, resumed, full = runs["first"]["rows"], runs["resumed"]["rows"], runs["full"]["rows"]
    assert first[-1, 1] <= 1e-6 and len(first) < len(full)
    # the resumed run starts where the first stopped, not from zero
    assert resumed[0, 1] < 1e-3 * full[0, 1]
    assert resumed[-1, 1] <= 1e-15
    for k in ("I", "Q", "U"):
        a = read_map(runs["resumed"]["names"][k])
        b = read_map(runs["full"]["names"][k])
        assert rel_rms(a, b, remove_monopole=(k == "I")) < 1e-6, k
    # the start map is the compact vector the first run wrote
    assert read_map(runs["first"]["names"]["A"]).size == read_map(runs["full"]["names"]["A"]).size
