"""Gain recalibration on the GPU (sg_set_gains / sg_fit_gains, sg_recal.cu;
the reference's -r / -R, sanepic.cc:1041-1130, 2123-2316) against the oracle
and the reference's own first gain fit, through the C ABI and the drop-in
executable."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
import sanepic_gb300 as sg
from golden_util import rel_rms
from sanepic_gb300 import build, synth
from test_recal_oracle import RECAL_TAGS, REF_FACTOR, recal_loop, recal_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


def problem(ndet, nseg=4, ns=4096, nside=16, precision="f64", problem=11, hwp=False):
    spec = synth.ProblemSpec("t", ndet=ndet, nside=nside, nseg=nseg, ns=ns, hwp=hwp,
                             fknee=0.05, alpha=1.0, problem=problem, precision=precision)
    return synth.make_problem(spec)


def comp_err(x, y, npix):
    return max(rel_rms(x[c * npix:(c + 1) * npix], y[c * npix:(c + 1) * npix],
                       remove_monopole=(c == 0)) for c in range(3))


@pytest.mark.parametrize("tag", RECAL_TAGS)
def test_first_fit_vs_reference(tag):
    """the map of the first loop (gains 1) and the fit to it: chi^2 before as
    the reference prints it, the per-detector coefficients it prints (/4,
    normalised to mean 1), and the oracle's fit to the GPU's own map"""
    prob, a1, log = recal_problem(tag)
    spec = prob["spec"]
    tod = prob["tod"].reshape(-1)
    mm = sg.from_problem(prob, precision="f64")
    mm.rhs()
    rep = mm.solve(precond="diag", stop_crit=1e-15, maxiter=2000)
    assert rep["converged"] and rep["crit0"] == 1.0  # x0 = 0: var0 = var00
    x = mm.solution()
    s = oracle.Setup(prob)
    assert comp_err(x, a1, s.npix) < 1e-6
    g, before, after = mm.fit_gains()
    assert before == pytest.approx(log["per_tile"]["before"], rel=1e-8)
    gd, before_d, after_d = mm.fit_gains(per_detector=True)
    coef = np.array(log["per_detector"]["coef"]) / REF_FACTOR
    np.testing.assert_allclose(gd[0], coef / coef.mean(), rtol=1e-6)
    assert np.ptp(gd, axis=0).max() == 0.0
    # the oracle's fit to the same map: the sums, the -R sums and chi^2
    ones = np.ones((spec.nseg, spec.ndet))
    for pdet, got in ((False, (g, before, after)), (True, (gd, before_d, after_d))):
        go, bo, ao = s.fit_gains(x, tod, ones, per_detector=pdet)
        np.testing.assert_allclose(got[0], go, rtol=1e-11)
        assert got[1] == pytest.approx(bo, rel=1e-11)
        assert got[2] == pytest.approx(ao, rel=1e-11)
        assert got[2] < got[1]


@pytest.mark.parametrize("prec,ndet", [("f64", 2), ("f64", 4), ("f32", 2), ("f32", 6)])
def test_operator_and_solve_with_gains_vs_oracle(prec, ndet):
    """A = P^T G N^-1 G P and b = P^T G N^-1 d tile by tile; ndet >= 4 on one
    pointing makes an offset-group context, which runs per detector while
    gains are set and returns to the group operator without them"""
    prob = problem(ndet, precision=prec)
    spec = prob["spec"]
    s = oracle.Setup(prob)
    mm = sg.from_problem(prob, precision=prec)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(3 * s.npix)
    g = 1.0 + 0.05 * rng.standard_normal((spec.nseg, spec.ndet))
    grouped = mm.weighting().startswith("group")
    assert grouped == (ndet >= 4)
    mm.set_gains(g)
    assert mm.weighting().startswith("per-detector")
    tol = 1e-11 if prec == "f64" else 1e-5
    assert rel_rms(mm.apply(x), s.apply_gains(x, g)) < tol
    # b with gains; chi^2_0 stays that of the raw data
    chi2 = mm.rhs()
    b_o = s.rhs_gains(prob["tod"], g)
    _, chi2_o = s.rhs(prob["tod"])
    assert chi2 == pytest.approx(chi2_o, rel=1e-10 if prec == "f64" else 1e-5)
    stop = 1e-14 if prec == "f64" else 1e-12
    rep = mm.solve(precond="bj3", stop_crit=stop, maxiter=1000)
    assert rep["converged"]
    xg = mm.solution()
    # the GPU's map in the oracle's system: |b - A x| / |b| over the entries
    # the solve keeps (the degeneracy mask zeroes the others)
    keep = ~oracle.masked(s)
    r = (b_o - s.apply_gains(xg, g))[keep]
    assert np.linalg.norm(r) / np.linalg.norm(b_o[keep]) < 10 * np.sqrt(stop)
    if prec == "f64":
        xo, _, _ = s.pcg_gains(b_o, g, precond="bj3", stop_crit=stop, maxiter=1000)
        assert comp_err(xg, xo, s.npix) < 1e-6
    # gains off: the group operator again (when the context has one)
    mm.set_gains(None)
    assert mm.weighting().startswith("group") == grouped
    assert rel_rms(mm.apply(x), s.apply(x)) < tol


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_recalibration_loop_vs_oracle(prec):
    """the outer loop (map with the gains, fit, repeat) on a problem with
    known gains, loop by loop against the oracle's"""
    spec = synth.ProblemSpec("recal_4det_nside16", ndet=4, nside=16, nseg=8, ns=2048,
                             fknee=0.02, alpha=1.0, problem=5, sigma_uk=5.0, precision=prec)
    prob = synth.make_problem(spec)
    gtrue = 1.0 + 0.02 * np.random.default_rng(2).standard_normal((4, 8))
    tod = prob["tod"].copy()
    for d in range(4):
        for sgi in range(8):
            tod[d, sgi * spec.ns:(sgi + 1) * spec.ns] *= gtrue[d, sgi]
    gp = dict(prob, tod=tod)
    mm = sg.from_problem(gp, precision=prec)
    nloop = 4
    g = np.ones((8, 4))
    x0 = None
    hist = []
    for _ in range(nloop):
        mm.set_gains(g)
        mm.rhs(chi2=False)
        rep = mm.solve(precond="diag", stop_crit=1e-15 if prec == "f64" else 1e-12,
                       maxiter=2000, x0=x0)
        assert rep["converged"]
        x0 = mm.solution()
        g, before, after = mm.fit_gains()
        hist.append((before, after))
    g_o, hist_o = recal_loop(prob, gtrue, nloop)
    rtol = 1e-7 if prec == "f64" else 1e-4
    np.testing.assert_allclose(g, g_o, rtol=rtol)
    np.testing.assert_allclose(np.array(hist), np.array(hist_o), rtol=rtol)
    chi = [h for pair in hist for h in pair]
    assert all(b <= a * (1 + 1e-9) for a, b in zip(chi, chi[1:]))


def test_recalibrate_loop_of_the_python_api():
    """MapMaker.recalibrate: the outer loop with its stop rule, loop by loop
    the oracle's (six loops here, the rule does not stop it earlier)"""
    spec = synth.ProblemSpec("recal_4det_nside16", ndet=4, nside=16, nseg=8, ns=2048,
                             fknee=0.02, alpha=1.0, problem=5, sigma_uk=5.0)
    prob = synth.make_problem(spec)
    gtrue = 1.0 + 0.02 * np.random.default_rng(2).standard_normal((4, 8))
    tod = prob["tod"].copy()
    for d in range(4):
        for sgi in range(8):
            tod[d, sgi * spec.ns:(sgi + 1) * spec.ns] *= gtrue[d, sgi]
    mm = sg.from_problem(dict(prob, tod=tod), precision="f64")
    out = mm.recalibrate(precond="diag", stop_crit=1e-15, max_loops=6)
    assert out["loops"] == 6 and len(out["chi2"]) == 6 and len(out["iterations"]) == 6
    g_o, hist_o = recal_loop(prob, gtrue, 6)
    np.testing.assert_allclose(out["gains"], g_o, rtol=1e-7)
    np.testing.assert_allclose(np.array(out["chi2"]), np.array(hist_o), rtol=1e-7)


def test_gain_arguments_and_learned_part_refused():
    prob = problem(2, nseg=2, ns=2048)
    mm = sg.from_problem(prob, precision="f64")
    bad = np.ones((2, 2))
    for v in (0.0, -1.0, np.nan, np.inf):
        bad[1, 0] = v
        with pytest.raises(sg.SanepicError):
            mm.set_gains(bad)
    with pytest.raises(sg.SanepicError):  # no map yet
        mm.fit_gains()
    mm.set_gains(np.full((2, 2), 1.01))
    with pytest.raises(sg.SanepicError):  # the training problems are made without gains
        mm.learn_train(npairs=8, steps=0)


CHI = re.compile(r"(Before|After) recal chi2 = (\S+)")


@pytest.mark.parametrize("glob", [False, True])
def test_cli_recalibration_loop(glob, tmp_path):
    """-r 1 (and -R 1): the outer loop of the drop-in executable on the
    reference's file tree: its first chi^2 as the reference prints it, the
    gains of relCalib.dat1 as the oracle fits them to the first map, chi^2
    falling loop after loop, one map set per loop, and an end before 500"""
    prob, _, log = recal_problem()
    spec = prob["spec"]
    args = synth.write_reference_tree(prob, str(tmp_path))
    for name in prob["names"]:
        np.zeros(spec.nseg * spec.ns).tofile(os.path.join(str(tmp_path), "tod_list",
                                                          f"orbdip_{name}"))
    args += ["-r", "1"] + (["-R", "1"] if glob else [])
    env = dict(os.environ, SANEPIC_GPU_PRECOND="diag", SANEPIC_GPU_PRECISION="f64")
    r = subprocess.run([build.CLI] + args, capture_output=True, text=True, timeout=900, env=env,
                       cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    chi = [(m.group(1), float(m.group(2))) for m in CHI.finditer(r.stdout)]
    nloops = len(chi) // 2
    assert 2 <= nloops < 500
    assert chi[0][1] == pytest.approx(log["per_tile"]["before"], rel=1e-8)
    vals = [v for _, v in chi]
    assert all(b <= a * (1 + 1e-9) for a, b in zip(vals, vals[1:]))
    if glob:
        assert len(re.findall(r"Coef calib det \d+ is", r.stdout)) == nloops * spec.ndet
    e = f"output_N{spec.nside}_.bin"
    out = os.path.join(str(tmp_path), "out_dir", "map_")
    a1 = np.fromfile(f"{out}_A_{e}_1", dtype="<f8")
    g1 = np.fromfile(os.path.join(str(tmp_path), "relCalib.dat1"), dtype="<f8")
    s = oracle.Setup(prob)
    go, _, _ = s.fit_gains(a1, prob["tod"].reshape(-1), np.ones((spec.nseg, spec.ndet)),
                           per_detector=glob)
    np.testing.assert_allclose(g1, go.reshape(-1), rtol=1e-11)
    for k in range(1, nloops + 1):
        for c in "AIQU":
            assert os.path.exists(f"{out}_{c}_{e}_{k}"), (c, k)
        assert os.path.exists(os.path.join(str(tmp_path), f"relCalib.dat{k}"))
    assert not os.path.exists(f"{out}_A_{e}_{nloops + 1}")


def test_cli_refuses_a_nonzero_orbital_dipole(tmp_path):
    prob, _, _ = recal_problem()
    spec = prob["spec"]
    args = synth.write_reference_tree(prob, str(tmp_path))
    dip = np.zeros(spec.nseg * spec.ns)
    dip[5] = 1e-6
    dip.tofile(os.path.join(str(tmp_path), "tod_list", f"orbdip_{prob['names'][0]}"))
    r = subprocess.run([build.CLI] + args + ["-r", "1"], capture_output=True, text=True,
                       timeout=300, cwd=str(tmp_path))
    assert r.returncode != 0 and "orbital dipole" in r.stderr
