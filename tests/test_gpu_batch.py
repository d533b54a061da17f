"""Batched solves of uneven independent problems and the FFT tile-shape
autotuner (GPU, through the C ABI)."""
import numpy as np
import pytest

import sanepic_gb300 as sg
from sanepic_gb300 import build, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


def _makers():
    specs = [synth.ProblemSpec("b0", ndet=2, nside=16, nseg=4, ns=4096, fknee=0.05, problem=41,
                               precision="f32"),
             synth.ProblemSpec("b1", ndet=4, nside=32, nseg=6, ns=16384, fknee=0.1, problem=42,
                               precision="f32"),
             synth.ProblemSpec("b2", ndet=2, nside=16, nseg=8, ns=2048, fknee=0.2, problem=43,
                               precision="f32"),
             synth.ProblemSpec("b3", ndet=3, nside=32, nseg=3, ns=32768, fknee=0.02, problem=44,
                               precision="f32")]
    out = []
    for s in specs:
        mm = sg.from_problem(synth.make_problem(s), precision="f32")
        mm.rhs()
        out.append(mm)
    return out


def test_batch_equals_individual_solves():
    makers = _makers()
    single = []
    for mm in makers:
        rep = mm.solve(precond="bj3", stop_crit=1e-10, maxiter=500)
        single.append((rep, mm.solution()))
    reps = sg.solve_batch(makers, precond="bj3", stop_crit=1e-10, maxiter=500)
    for (rep1, x1), rep2, mm in zip(single, reps, makers):
        assert rep1["converged"], rep1
        assert rep2["converged"] and rep2["iterations"] == rep1["iterations"], (rep1, rep2)
        # same kernels, same order, fixed-order reductions: the same bits
        assert np.array_equal(mm.solution(), x1)


def test_batch_rejects_missing_rhs():
    spec = synth.ProblemSpec("nr", ndet=1, nside=16, nseg=2, ns=2048, problem=45, precision="f32")
    mm = sg.from_problem(synth.make_problem(spec), precision="f32")
    with pytest.raises(sg.SanepicError):
        sg.solve_batch([mm], precond="bj3")


def test_autotune_keeps_the_operator():
    spec = synth.ProblemSpec("at", ndet=2, nside=32, nseg=4, ns=32768, fknee=0.1, problem=46,
                             precision="f32")
    mm = sg.from_problem(synth.make_problem(spec), precision="f32")
    x = np.random.default_rng(3).standard_normal(3 * mm.npix)
    y0 = mm.apply(x)
    t = mm.autotune()
    assert t["cluster_size"] in (2, 4) and t["filter_ms"] > 0
    assert t["pt_lanes"] in (1, 2, 4, 8, 16, 32)
    y1 = mm.apply(x)
    assert np.linalg.norm(y1 - y0) <= 1e-5 * np.linalg.norm(y0)
    mm.rhs()
    assert mm.solve(precond="bj3", stop_crit=1e-10)["converged"]


def test_autotuned_pt_team_is_deterministic():
    """whatever lane team the autotuner keeps for P^T, A x is the same map
    (FP32 sums in another order) and is bitwise repeatable"""
    spec = synth.ProblemSpec("atp", ndet=3, nside=64, nseg=4, ns=16384, fknee=0.1, problem=49,
                             precision="f32")
    mm = sg.from_problem(synth.make_problem(spec), precision="f32")
    x = np.random.default_rng(5).standard_normal(3 * mm.npix)
    y0 = mm.apply(x)
    mm.autotune()
    y1, y2 = mm.apply(x), mm.apply(x)
    assert np.array_equal(y1, y2)
    assert np.linalg.norm(y1 - y0) <= 1e-5 * np.linalg.norm(y0)


def test_autotune_keeps_the_group_operator():
    """co-pointed detectors run the offset-group operator, whose spectra are
    stored in the slot order of the tile shape: a changed shape rebuilds the
    mixing matrices and A stays the same map"""
    spec = synth.ProblemSpec("atg", ndet=8, nside=32, nseg=4, ns=32768, fknee=0.1, problem=47,
                             precision="f32")
    mm = sg.from_problem(synth.make_problem(spec), precision="f32")
    assert mm.group_mode()[0]
    x = np.random.default_rng(4).standard_normal(3 * mm.npix)
    y0 = mm.apply(x)
    t = mm.autotune()
    assert t["cluster_size"] in (2, 4) and t["filter_ms"] > 0
    y1 = mm.apply(x)
    assert np.linalg.norm(y1 - y0) <= 1e-5 * np.linalg.norm(y0)
    mm.rhs()
    assert mm.solve(precond="bj3", stop_crit=1e-10)["converged"]


def test_autotune_needs_the_noise():
    """the autotuner times the operator, so it refuses a context without
    every detector's noise spectrum"""
    spec = synth.ProblemSpec("atn", ndet=2, nside=16, nseg=2, ns=2048, problem=48, precision="f32")
    prob = synth.make_problem(spec)
    mm = sg.MapMaker(spec.ns, spec.nseg, spec.ndet, spec.nside, precision="f32")
    mm.set_pointing(prob["ra"], prob["dec"], prob["psi"], sg.detectors_from_angles(prob["angles"]),
                    prob.get("isampmin"))
    mm.set_noise(0, prob["ispf"][0])
    with pytest.raises(sg.SanepicError):
        mm.autotune()
    mm.set_noise(1, prob["ispf"][1])
    assert mm.autotune()["cluster_size"] >= 1
