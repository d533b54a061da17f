"""GPU parity: libsanepic_gpu (called through the C ABI) against the CPU
oracle and the reference's own outputs (tests/golden)."""
import numpy as np
import pytest

import oracle
import sanepic_gb300 as sg
from sanepic_gb300 import build
from golden_util import NAMES, load_log, load_outputs, load_problem, rel_rms
from sanepic_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


def small_problem(ndet=2, nside=16, nseg=4, ns=2048, hwp=False, problem=7, fknee=0.1,
                  precision="f64"):
    spec = synth.ProblemSpec("t", ndet=ndet, nside=nside, nseg=nseg, ns=ns, hwp=hwp,
                             fknee=fknee, alpha=1.0, problem=problem, precision=precision)
    return synth.make_problem(spec)


# ---- pixelisation -------------------------------------------------------------
@pytest.mark.parametrize("name", NAMES)
def test_pixels_bit_exact(name):
    prob = load_problem(name)
    mm = sg.from_problem(prob, precision="f64")
    s = oracle.Setup(prob)
    assert np.array_equal(mm.pixels(), s.pix)
    assert np.array_equal(mm.indpix(), s.indpix)
    assert mm.npix == s.npix


def test_pixels_bit_exact_1det_nside64_full_size():
    spec = synth.spec_from_name("c1_1det_nside64")
    prob = synth.make_problem(spec, with_tod=False)
    mm = sg.from_problem(prob, with_tod=False)
    s = oracle.Setup(prob)
    assert np.array_equal(mm.pixels(), s.pix)


def test_pixels_with_detector_offsets_and_hwp():
    prob = small_problem(ndet=3, hwp=True)
    offs = [(0.0, 0.0), (0.01, -0.02), (0.01, -0.02)]
    mm = sg.MapMaker(prob["spec"].ns, prob["spec"].nseg, 3, prob["spec"].nside, hwp=True,
                     omega=prob["omega"], precision="f64")
    mm.set_pointing(prob["ra"], prob["dec"], prob["psi"],
                    sg.detectors_from_angles(prob["angles"], offs))
    s = oracle.Setup(prob, det_offsets=offs)
    assert np.array_equal(mm.pixels(), s.pix)


@pytest.mark.parametrize("name", NAMES)
def test_reference_hits_and_weights(name):
    prob = load_problem(name)
    ref = load_outputs(name)
    mm = sg.from_problem(prob, precision="f64")
    assert np.array_equal(mm.get_map("HITS"), ref["HITS"])
    assert np.array_equal(mm.get_map("POL_HITS"), ref["POL_HITS"])
    for k in ("COS2P", "SIN2P", "NVAR", "Q_NVAR", "U_NVAR"):
        assert rel_rms(mm.get_map(k), ref[k]) < 1e-10, k


def test_cross_link_maps_same_in_both_precisions():
    """COS2P/SIN2P are FP64 sums whatever the operator precision (without a
    half-wave plate their cos/sin come from the base-angle pass's FP64 table)"""
    prob = small_problem(ndet=4, nseg=2, ns=4096, nside=32)
    m64 = sg.from_problem(prob, precision="f64", with_tod=False)
    m32 = sg.from_problem(prob, precision="f32", with_tod=False)
    for k in ("COS2P", "SIN2P"):
        assert np.array_equal(m64.get_map(k), m32.get_map(k)), k


# ---- noise filter (FFT) ---------------------------------------------------------
@pytest.mark.parametrize("ns,prec", [(256, "f64"), (2048, "f64"), (16384, "f64"),
                                     (65536, "f64"), (1024, "f32"), (32768, "f32"),
                                     (131072, "f32")])
def test_noise_filter_vs_oracle(ns, prec):
    prob = small_problem(ndet=2, nseg=2, ns=ns, precision=prec)
    s = oracle.Setup(prob)
    mm = sg.from_problem(prob, precision=prec, with_tod=False)
    rng = np.random.default_rng(ns)
    x = rng.standard_normal(2 * 2 * ns)
    got = mm.noise_filter(x)
    want = np.concatenate([s.noise_filter(d, x[(d * 2 + g) * ns:(d * 2 + g + 1) * ns])
                           for d in range(2) for g in range(2)])
    tol = 1e-12 if prec == "f64" else 2e-6
    assert rel_rms(got, want) < tol


@pytest.mark.parametrize("ns", [4096, 131072])
def test_noise_filter_vs_cufft(ns):
    # the hand-written cluster FFT filter (FP32) against cuFFT in FP64
    # (torch.fft): y = c2r(h . r2c(x)) with FFTW's unnormalised scaling and
    # the weights of sanepic.cc:533-537 -- cuFFT only as a cross-check
    torch = pytest.importorskip("torch")
    prob = small_problem(ndet=2, nseg=3, ns=ns, precision="f32")
    mm = sg.from_problem(prob, precision="f32", with_tod=False)
    x = np.random.default_rng(ns + 1).standard_normal(2 * 3 * ns)
    got = mm.noise_filter(x)
    k = np.arange(ns // 2 + 1, dtype=np.float64)
    want = []
    for d in range(2):
        ispf = prob["ispf"][d]
        h = ispf[(k / ispf.size * ns).astype(np.int64)] / ns / ns
        h[0] = ispf[1] * 1e-6 / ns / ns
        xt = torch.tensor(x[d * 3 * ns:(d + 1) * 3 * ns].reshape(3, ns), dtype=torch.float64,
                          device="cuda")
        ht = torch.tensor(h, dtype=torch.float64, device="cuda")
        yt = torch.fft.irfft(torch.fft.rfft(xt, dim=1) * ht, n=ns, dim=1) * ns
        want.append(yt.cpu().numpy().reshape(-1))
    want = np.concatenate(want)
    assert rel_rms(got, want) < 2e-6


def test_noise_of_every_detector_in_one_call():
    """sg_set_noise_all makes the rows sg_set_noise makes, detector by detector"""
    prob = small_problem(ndet=3, nseg=2, ns=4096, precision="f32", nside=16)
    one = sg.from_problem(prob, precision="f32")
    allm = sg.from_problem(prob, precision="f32")
    allm.set_noise_all(np.asarray(prob["ispf"]))
    x = np.random.default_rng(4).standard_normal(3 * one.npix)
    assert np.array_equal(one.apply(x), allm.apply(x))
    assert one.rhs() == allm.rhs()
    with pytest.raises(ValueError):
        allm.set_noise_all(np.asarray(prob["ispf"])[:2])
    # and every detector's timeline in one call, one of them with NaNs
    tod = np.array(prob["tod"], dtype=np.float64)
    tod[1, 100] = np.nan
    tod[2, 4096 + 7] = np.nan
    for d in range(3):
        one.set_tod(d, tod[d])
    allm.set_tod_all(tod)
    assert one.rhs() == allm.rhs()
    one.solve(precond="bj3", stop_crit=1e-10)
    allm.solve(precond="bj3", stop_crit=1e-10)
    assert np.array_equal(one.solution(), allm.solution())


# ---- operator ---------------------------------------------------------------------
# ndet >= 4 on one pointing: the offset-group operator (three timelines per
# group, 3 x 3 spectral mixing); ndet = 2: one filter per detector
@pytest.mark.parametrize("prec,ns,ndet,hwp", [("f64", 2048, 2, False), ("f64", 65536, 2, False),
                                              ("f32", 4096, 2, False), ("f32", 131072, 2, False),
                                              ("f64", 4096, 4, False), ("f64", 2048, 6, True),
                                              ("f32", 4096, 8, False), ("f32", 131072, 8, True)])
def test_apply_vs_oracle(prec, ns, ndet, hwp):
    nseg = 2 if ns >= 65536 else 4
    prob = small_problem(ndet=ndet, nseg=nseg, ns=ns, precision=prec, nside=32, hwp=hwp)
    s = oracle.Setup(prob)
    mm = sg.from_problem(prob, precision=prec, with_tod=False)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(3 * s.npix)
    got = mm.apply(x)
    want = s.apply(x)
    tol = 1e-11 if prec == "f64" else 1e-5
    assert rel_rms(got, want) < tol
    # A is symmetric: x^T A y = y^T A x
    y = rng.standard_normal(3 * s.npix)
    a, b = x @ mm.apply(y), y @ mm.apply(x)
    assert abs(a - b) <= (1e-10 if prec == "f64" else 1e-5) * max(abs(a), abs(b))


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_group_operator_matches_per_detector(prec, monkeypatch):
    """the offset-group operator and the per-detector one are the same linear
    map: A x agrees to rounding, and so do the solves"""
    prob = small_problem(ndet=8, nseg=4, ns=8192, precision=prec, nside=32, hwp=True)
    x = np.random.default_rng(5).standard_normal(3 * oracle.Setup(prob).npix)
    grouped = sg.from_problem(prob, precision=prec)
    monkeypatch.setenv("SANEPIC_GPU_GROUP_FILTER", "0")
    per_det = sg.from_problem(prob, precision=prec)
    tol = 1e-12 if prec == "f64" else 2e-6
    assert rel_rms(grouped.apply(x), per_det.apply(x)) < tol
    for mm in (grouped, per_det):
        mm.rhs()
    a = grouped.solve(precond="bj3", stop_crit=1e-12)
    xa = grouped.solution()
    b = per_det.solve(precond="bj3", stop_crit=1e-12)
    xb = per_det.solution()
    assert a["converged"] and b["converged"] and abs(a["iterations"] - b["iterations"]) <= 1
    npix = grouped.npix
    assert rel_rms(xa[npix:], xb[npix:]) < (1e-7 if prec == "f64" else 1e-4)


@pytest.mark.parametrize("ns,distinct,hwp,nseg", [(2048, True, False, 4), (16384, False, True, 5),
                                                  (65536, True, True, 5), (131072, True, False, 3),
                                                  (131072, False, False, 4)])
def test_three_pass_weighting_vs_cluster_kernels_and_oracle(ns, distinct, hwp, nseg, monkeypatch):
    """the three-pass FP32 group weighting (sg_fft3.cu, in place in P^T's
    layout) and the cluster FFT kernels are the same operator: A x of both
    against the oracle and against each other; segment counts that do not
    fill the row kernel's 3-segment blocks included"""
    spec = synth.ProblemSpec("t", ndet=6, nside=32, nseg=nseg, ns=ns, hwp=hwp,
                             fknee_range=(0.02, 0.2) if distinct else None,
                             alpha_range=(1.0, 2.0) if distinct else None,
                             fknee=0.1, alpha=1.0, problem=23, precision="f32")
    prob = synth.make_problem(spec, with_tod=False)
    s = oracle.Setup(prob)
    x = np.random.default_rng(4).standard_normal(3 * s.npix)
    f3 = sg.from_problem(prob, precision="f32", with_tod=False)
    y3 = f3.apply(x)
    assert f3.weighting() == "group-3pass"
    monkeypatch.setenv("SANEPIC_GPU_FFT3", "0")
    cl = sg.from_problem(prob, precision="f32", with_tod=False)
    yc = cl.apply(x)
    assert cl.weighting() == "group"
    yo = s.apply(x)
    assert rel_rms(y3, yo) < 1e-5
    assert rel_rms(yc, yo) < 1e-5
    assert rel_rms(y3, yc) < 2e-6
    # symmetric, and deterministic run to run
    z = np.random.default_rng(5).standard_normal(3 * s.npix)
    a, b = z @ f3.apply(x), x @ f3.apply(z)
    assert abs(a - b) <= 1e-5 * max(abs(a), abs(b))
    assert np.array_equal(f3.apply(x), y3)
    f3.close()
    cl.close()


@pytest.mark.parametrize("ns,hwp", [(8192, False), (131072, True)])
def test_three_pass_rhs_vs_cluster_kernels_and_oracle(ns, hwp, monkeypatch):
    """the right-hand side of groups with distinct noise spectra through the
    three-pass forward FFT (batched column and row passes, half spectra in
    position order), the group sums and the three-pass inverse: chi^2_0 and
    the solution against the oracle and against the cluster kernels"""
    spec = synth.ProblemSpec("t", ndet=6, nside=32, nseg=3, ns=ns, hwp=hwp,
                             fknee_range=(0.02, 0.2), alpha_range=(1.0, 2.0), problem=29,
                             precision="f32")
    prob = synth.make_problem(spec)
    s = oracle.Setup(prob)
    b, chi2o = s.rhs(prob["tod"])
    xo, _, _ = s.pcg(b, precond="bj3", stop_crit=1e-15, maxiter=500)
    out = {}
    for f3 in ("1", "0"):
        monkeypatch.setenv("SANEPIC_GPU_FFT3", f3)
        mm = sg.from_problem(prob, precision="f32")
        chi2 = mm.rhs()
        mm.solve(precond="bj3", stop_crit=1e-14)
        out[f3] = (chi2, mm.solution(), mm.weighting())
        npix = mm.npix
        mm.close()
    assert out["1"][2] == "group-3pass" and out["0"][2] == "group"
    for f3, (chi2, x, _) in out.items():
        assert abs(chi2 - chi2o) <= 1e-5 * chi2o, f3
        for c in range(3):
            blk = slice(c * npix, (c + 1) * npix)
            assert rel_rms(x[blk], xo[blk], remove_monopole=(c == 0)) < 1e-5, (f3, c)
    for c in range(3):
        blk = slice(c * npix, (c + 1) * npix)
        assert rel_rms(out["1"][1][blk], out["0"][1][blk], remove_monopole=(c == 0)) < 2e-6, c


@pytest.mark.parametrize("ns,nseg,hwp", [(4096, 5, False), (131072, 49, True)])
def test_three_pass_detector_filter_vs_cluster_kernels_and_oracle(ns, nseg, hwp, monkeypatch):
    """the per-detector operator (three co-pointed detectors: fewer than an
    offset group needs) with the three-pass FP32 filter (batches through L2;
    at 131072 samples 147 tiles cross a 96-tile batch boundary and leave a
    partial 4-tile row block) against the cluster filter and the oracle; the
    right-hand side without chi^2 takes the same filter (out of place), and
    the small case's solution is checked against the oracle's"""
    spec = synth.ProblemSpec("t", ndet=3, nside=32, nseg=nseg, ns=ns, hwp=hwp,
                             fknee_range=(0.02, 0.2), alpha_range=(1.0, 2.0), problem=31,
                             precision="f32")
    prob = synth.make_problem(spec)
    s = oracle.Setup(prob)
    x = np.random.default_rng(6).standard_normal(3 * s.npix)
    f3 = sg.from_problem(prob, precision="f32")
    y3 = f3.apply(x)
    assert f3.weighting() == "per-detector-3pass"
    monkeypatch.setenv("SANEPIC_GPU_FFT3", "0")
    cl = sg.from_problem(prob, precision="f32")
    yc = cl.apply(x)
    assert cl.weighting() == "per-detector"
    cl.close()
    yo = s.apply(x)
    assert rel_rms(y3, yo) < 1e-5
    assert rel_rms(yc, yo) < 1e-5
    assert rel_rms(y3, yc) < 2e-6
    if ns <= 4096:
        assert f3.rhs(chi2=False) is None
        rep = f3.solve(precond="bj3", stop_crit=1e-14)
        assert rep["converged"]
        x3 = f3.solution()
        b, _ = s.rhs(prob["tod"])
        xo, _, _ = s.pcg(b, precond="bj3", stop_crit=1e-15, maxiter=500)
        npix = s.npix
        for c in range(3):
            blk = slice(c * npix, (c + 1) * npix)
            assert rel_rms(x3[blk], xo[blk], remove_monopole=(c == 0)) < 1e-5, c
    f3.close()


def test_apply_bitwise_deterministic():
    prob = small_problem(ndet=4, nseg=4, ns=4096, precision="f32", nside=32)
    mm = sg.from_problem(prob, precision="f32", with_tod=False)
    x = np.random.default_rng(3).standard_normal(3 * mm.npix)
    y1, y2 = mm.apply(x), mm.apply(x)
    assert np.array_equal(y1, y2)


@pytest.mark.parametrize("name", NAMES)
def test_rhs_and_solution_vs_reference(name):
    prob = load_problem(name)
    ref = load_outputs(name)
    log = load_log(name)
    mm = sg.from_problem(prob, precision="f64")
    mm.rhs()
    rep = mm.solve(precond="diag", stop_crit=1e-15, maxiter=2000)
    crit = mm.crit_history()
    ref_crit = np.array([c[1] for c in log["crit"]])
    n = min(10, len(ref_crit))
    np.testing.assert_allclose(crit[:n], ref_crit[:n], rtol=1e-6)
    assert abs(rep["iterations"] - log["iterations"]) <= max(3, log["iterations"] // 10)
    assert rel_rms(mm.get_map("I"), ref["I"], remove_monopole=True) < 1e-6
    assert rel_rms(mm.get_map("Q"), ref["Q"]) < 1e-6
    assert rel_rms(mm.get_map("U"), ref["U"]) < 1e-6


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_bj3_solve_vs_oracle(prec):
    prob = small_problem(ndet=4, nseg=8, ns=4096, precision=prec, nside=16, fknee=0.05)
    s = oracle.Setup(prob)
    b, _ = s.rhs(prob["tod"])
    mm = sg.from_problem(prob, precision=prec)
    mm.rhs()
    # same stopping point on both sides (|r|/|b| = 1e-6), then a deeper one
    checks = [(1e-12, 1e-5)] + ([(1e-14, 1e-6)] if prec == "f64" else [])
    for stop, tol in checks:
        xo, it_o, _ = s.pcg(b, precond="bj3", stop_crit=stop, maxiter=500)
        rep = mm.solve(precond="bj3", stop_crit=stop, maxiter=500)
        assert rep["converged"]
        assert abs(rep["iterations"] - it_o) <= 2
        x = mm.solution()
        npix = s.npix
        for c in range(3):
            blk = slice(c * npix, (c + 1) * npix)
            err = rel_rms(x[blk], xo[blk], remove_monopole=(c == 0))
            assert err < tol, (stop, c, err)


def test_graph_and_eager_agree():
    prob = small_problem(ndet=2, nseg=4, ns=2048, precision="f32")
    mm = sg.from_problem(prob, precision="f32")
    mm.rhs()
    mm.solve(precond="bj3", stop_crit=1e-8, use_graph=True)
    a = mm.solution()
    mm.solve(precond="bj3", stop_crit=1e-8, use_graph=False)
    b = mm.solution()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_tod_nan_rule_matches_reference(prec):
    """NaN samples take the previous sample's value within their segment
    (sanepic.cc:784-790); the library applies the rule on the GPU."""
    prob = small_problem(ndet=2, nseg=4, ns=2048, precision=prec)
    ns = prob["spec"].ns
    tod_nan = [t.copy() for t in prob["tod"]]
    rng = np.random.default_rng(8)
    for t in tod_nan:
        for i in rng.integers(1, t.size, 40):
            if i % ns:                              # not a segment's first sample
                t[i:i + rng.integers(1, 5)] = np.nan  # runs, some across segments
    tod_ref = [t.copy() for t in tod_nan]
    for t in tod_ref:                               # the reference's rule, on the host
        for g in range(prob["spec"].nseg):
            s = t[g * ns:(g + 1) * ns]
            for i in range(1, ns):
                if np.isnan(s[i]):
                    s[i] = s[i - 1]
    out = []
    for tods in (tod_nan, tod_ref):
        p = dict(prob, tod=tods)
        mm = sg.from_problem(p, precision=prec)
        chi2 = mm.rhs()
        mm.solve(precond="bj3", stop_crit=1e-8)
        out.append((chi2, mm.solution()))
        mm.close()
    assert np.isfinite(out[0][0]) and out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_tod_from_pinned_memory(prec):
    """timelines and noise spectra in pinned (page-locked) host memory are
    read by the kernels directly; the result equals the staged copy of
    ordinary memory, NaN rule included"""
    torch = pytest.importorskip("torch")
    prob = small_problem(ndet=4, nseg=4, ns=2048, precision=prec)
    tods = [t.copy() for t in prob["tod"]]
    tods[1][100:103] = np.nan
    out = []
    for pinned in (False, True):
        mm = sg.from_problem(dict(prob, tod=tods), precision=prec)
        if pinned:
            for d, t in enumerate(tods):
                buf = torch.empty(t.size, dtype=torch.float64, pin_memory=True)
                buf.numpy()[:] = t
                mm.set_tod(d, buf.numpy())
                nb = torch.empty(prob["ispf"][d].size, dtype=torch.float64, pin_memory=True)
                nb.numpy()[:] = prob["ispf"][d]
                mm.set_noise(d, nb.numpy())
        out.append((mm.rhs(), mm.solve(precond="bj3", stop_crit=1e-8)["iterations"],
                    mm.solution()))
        mm.close()
    assert np.isfinite(out[0][0]) and out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])


def test_psi_nan_rule_matches_oracle():
    """NaN boresight angles take the previous sample's psi within their segment
    (sanepic.cc:722-727, applied on the GPU): pixels and A x match the oracle"""
    prob = small_problem(ndet=4, nseg=4, ns=2048, precision="f64")
    ns = prob["spec"].ns
    psi = prob["psi"].copy()
    rng = np.random.default_rng(12)
    for i in rng.integers(1, psi.size - 8, 30):
        if i % ns and (i + 4) // ns == i // ns:    # inside one segment, not its first sample
            psi[i:i + rng.integers(1, 4)] = np.nan
    p = dict(prob, psi=psi)
    s = oracle.Setup(p)
    mm = sg.from_problem(p, precision="f64", with_tod=False)
    assert np.array_equal(mm.pixels(), s.pix)
    x = np.random.default_rng(2).standard_normal(3 * s.npix)
    assert rel_rms(mm.apply(x), s.apply(x)) < 1e-11


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_device_loop_matches_host_loop(prec, monkeypatch):
    """the PCG loop as one graph launch (a conditional WHILE node) runs the same
    kernels in the same order as the host-driven loop: identical iterations,
    crit history and map"""
    prob = small_problem(ndet=4, nseg=4, ns=4096, precision=prec, nside=16, fknee=0.05)
    out = []
    for env in ("1", "0"):
        monkeypatch.setenv("SANEPIC_GPU_DEVICE_LOOP", env)
        mm = sg.from_problem(prob, precision=prec)
        mm.rhs()
        rep = mm.solve(precond="bj3", stop_crit=1e-12, maxiter=300)
        out.append((rep["iterations"], mm.crit_history(), mm.solution()))
        # an iteration limit is honoured on the device as on the host
        lim = mm.solve(precond="bj3", stop_crit=1e-30, maxiter=7)
        assert lim["iterations"] == 7 and not lim["converged"]
        mm.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("hwp", [False, True])
def test_rhs_without_chi2_sums_detectors_with_one_noise_spectrum(hwp):
    # every detector with the same iSpf: without chi2_0 the right-hand side
    # sums the group's timelines before the FFTs; the map is the same
    prob = small_problem(ndet=6, nside=32, nseg=4, ns=8192, precision="f32", hwp=hwp)
    mm = sg.from_problem(prob, precision="f32")
    assert mm.group_mode()[0]
    chi2 = mm.rhs()
    assert chi2 > 0
    mm.solve(precond="bj3", stop_crit=1e-14)
    x1 = mm.solution()
    assert mm.rhs(chi2=False) is None
    mm.solve(precond="bj3", stop_crit=1e-14)
    x2 = mm.solution()
    npix = mm.npix
    s = oracle.Setup(prob)
    b, _ = s.rhs(prob["tod"])
    xo, _, _ = s.pcg(b, precond="bj3", stop_crit=1e-15, maxiter=500)
    for c in range(3):
        blk = slice(c * npix, (c + 1) * npix)
        assert rel_rms(x2[blk], x1[blk], remove_monopole=(c == 0)) < 1e-5, c
        assert rel_rms(x2[blk], xo[blk], remove_monopole=(c == 0)) < 1e-5, c


@pytest.mark.parametrize("prec,hwp", [("f64", False), ("f32", True)])
def test_group_operator_with_distinct_noise_spectra_vs_oracle(prec, hwp):
    # co-pointed detectors each with its own 1/f spectrum: the group operator
    # mixes the three timelines' spectra by a 3 x 3 matrix per frequency (with
    # one shared spectrum it mixes them in the time domain instead; the
    # uniform case is what the other operator tests run)
    spec = synth.ProblemSpec("t", ndet=6, nside=32, nseg=2, ns=8192, hwp=hwp,
                             fknee_range=(0.02, 0.2), alpha_range=(1.0, 2.0), problem=17,
                             precision=prec)
    prob = synth.make_problem(spec)
    s = oracle.Setup(prob)
    mm = sg.from_problem(prob, precision=prec, with_tod=False)
    assert mm.group_mode()[0]
    x = np.random.default_rng(2).standard_normal(3 * s.npix)
    tol = 1e-11 if prec == "f64" else 1e-5
    assert rel_rms(mm.apply(x), s.apply(x)) < tol
