"""The oracle's gain recalibration (sanepic.cc:2123-2316, 3206-3260) against
the reference's own first gain fit (tests/golden/recal_*_ref.*, made by
tests/golden/make_recal_golden.py: 4 detectors, and 2 with a half-wave
plate), and its corrected outer loop on a problem with known gains.

The reference's fit returns four times the least-squares gain (sPNd carries
a factor 2, cPNPc a factor 1/2); the fixture's numbers are checked with that
factor put back, so the pin covers every other step of the fit."""
import json
import os

import numpy as np
import pytest

import oracle
from golden_util import GOLDEN_DIR, load_problem
from sanepic_gb300 import synth

REF_FACTOR = 4.0  # sanepic.cc:2196-2201 (x 2) over 2217-2220 (x 1/2)


RECAL_TAGS = ["4det_nside16", "2det_nside16_hwp"]


def recal_problem(tag="4det_nside16"):
    z = np.load(os.path.join(GOLDEN_DIR, f"recal_{tag}_ref.npz"))
    with open(os.path.join(GOLDEN_DIR, f"recal_{tag}_ref.json")) as f:
        log = json.load(f)
    prob = load_problem(log["problem"])
    spec = prob["spec"]
    g = z["gains"]
    tod = prob["tod"].copy()
    for d in range(spec.ndet):
        for s in range(spec.nseg):
            tod[d, s * spec.ns:(s + 1) * spec.ns] *= g[d, s]
    prob["tod"] = tod
    return prob, z["A_1"], log


@pytest.mark.parametrize("tag", RECAL_TAGS)
def test_gain_fit_matches_the_references_first_fit(tag):
    prob, a1, log = recal_problem(tag)
    spec = prob["spec"]
    s = oracle.Setup(prob)
    tod = prob["tod"].reshape(-1)
    assert a1.size == 3 * s.npix
    # chi^2 with the gains the first map was made with (all 1)
    assert s.gain_chi2(a1, tod) == pytest.approx(log["per_tile"]["before"], rel=1e-12)
    bd, cs = s.gain_dots(a1, tod)  # [det][seg]
    # -r: one gain per tile; the reference's chi^2 with its (x4) gains
    g_tile = REF_FACTOR * bd / cs
    assert s.gain_chi2(a1, tod, g_tile.T) == pytest.approx(log["per_tile"]["after"], rel=1e-12)
    # -R: one gain per detector, printed as "Coef calib det"
    g_det = REF_FACTOR * bd.sum(axis=1) / cs.sum(axis=1)
    np.testing.assert_allclose(g_det, log["per_detector"]["coef"], rtol=1e-12)
    gd = np.repeat(g_det[None, :], spec.nseg, axis=0)
    assert s.gain_chi2(a1, tod, gd) == pytest.approx(log["per_detector"]["after"], rel=1e-12)


def test_fit_normalises_to_the_previous_mean_gain():
    prob, a1, _ = recal_problem()
    s = oracle.Setup(prob)
    tod = prob["tod"].reshape(-1)
    g0 = np.full((prob["spec"].nseg, prob["spec"].ndet), 1.1)
    g, before, after = s.fit_gains(a1, tod, g0)
    assert g.mean() == pytest.approx(1.1, rel=1e-14)
    gd, _, _ = s.fit_gains(a1, tod, g0, per_detector=True)
    assert np.ptp(gd, axis=0).max() == 0.0  # one gain per detector
    assert gd.mean() == pytest.approx(1.1, rel=1e-14)


def recal_loop(prob, gtrue, nloop, per_detector=False):
    spec = prob["spec"]
    tod = prob["tod"].copy()
    for d in range(spec.ndet):
        for s in range(spec.nseg):
            tod[d, s * spec.ns:(s + 1) * spec.ns] *= gtrue[d, s]
    st = oracle.Setup(prob)
    tod = tod.reshape(-1)
    g = np.ones((spec.nseg, spec.ndet))
    x = None
    Mp = st.diag_precond()
    hist = []
    for _ in range(nloop):
        b = st.rhs_gains(tod, g)
        x, _, _ = st.pcg_gains(b, g, precond="diag", x0=x, stop_crit=1e-15, Mp=Mp)
        g, before, after = st.fit_gains(x, tod, g, per_detector=per_detector)
        hist.append((before, after))
    return g, hist


@pytest.mark.parametrize("per_detector", [False, True])
def test_corrected_loop_recovers_the_injected_gains(per_detector):
    spec = synth.ProblemSpec("recal_4det_nside16", ndet=4, nside=16, nseg=8, ns=2048,
                             fknee=0.02, alpha=1.0, problem=5, sigma_uk=5.0)
    prob = synth.make_problem(spec)
    rng = np.random.default_rng(2)
    if per_detector:
        gtrue = np.repeat(1.0 + 0.02 * rng.standard_normal((4, 1)), 8, axis=1)
    else:
        gtrue = 1.0 + 0.02 * rng.standard_normal((4, 8))
    # one gain per detector is nearly degenerate with Q and U (a gain
    # mismatch between detectors at different angles looks like
    # polarisation), so that loop converges more slowly
    g, hist = recal_loop(prob, gtrue, 32 if per_detector else 6, per_detector)
    # chi^2 never rises: each fit lowers it, and each map made with the new
    # gains lowers it again
    chi = [h for pair in hist for h in pair]
    assert all(b <= a * (1 + 1e-12) for a, b in zip(chi, chi[1:]))
    # the gains up to the common factor the map absorbs: from 2 % off to
    # below 0.5 %, the noise floor of this problem
    ratio = g.T / gtrue
    assert np.std(ratio / ratio.mean()) < 0.005


def tile_sums(s, x, tod):
    """The per-tile sums sg_fit_gains forms on the GPU, here on the host from
    the oracle's pieces: (N^-1 d)^T s and (N^-1 s)^T s in the time domain
    (s = P x), and the bins 0 and ns/2 of s and d."""
    import ctypes
    L = oracle.lib()
    ns, nseg, ndet = s.ns, s.nseg, s.ndet
    dots_ds = np.empty((ndet, nseg))
    dots_ss = np.empty((ndet, nseg))
    edges_s = np.empty((ndet, nseg, 2))
    edges_d = np.empty((ndet, nseg, 2))
    sign = np.where(np.arange(ns) % 2 == 0, 1.0, -1.0)
    xs = np.ascontiguousarray(x, np.float64)
    for d in range(ndet):
        for g in range(nseg):
            off = ns * g + ns * nseg * d
            pv = np.empty(ns)
            L.orc_deproject(oracle._pd(xs), oracle._pl(s.indpix),
                            oracle._pl(np.ascontiguousarray(s.pix[off:off + ns])),
                            oracle._pd(np.ascontiguousarray(s.psip[off:off + ns])),
                            ctypes.c_long(ns), ctypes.c_long(s.npix), oracle._pd(pv))
            dv = tod[off:off + ns]
            dots_ds[d, g] = s.noise_filter(d, dv) @ pv
            dots_ss[d, g] = s.noise_filter(d, pv) @ pv
            edges_s[d, g] = (pv.sum(), sign @ pv)
            edges_d[d, g] = (dv.sum(), sign @ dv)
    spn_edge = np.stack([s.spn[np.arange(ndet) * ns], s.spn[np.arange(ndet) * ns + ns // 2]], 1)
    return dots_ds, dots_ss, edges_s, edges_d, spn_edge


@pytest.mark.parametrize("per_detector", [False, True])
def test_library_gain_arithmetic_matches_the_oracle_fit(per_detector):
    """the library's host arithmetic (sg_gains_from_sums) on time-domain sums
    plus the bins 0 and ns/2 gives the oracle's half-spectrum fit"""
    import sanepic_gb300 as sg
    prob, a1, _ = recal_problem()
    s = oracle.Setup(prob)
    tod = prob["tod"].reshape(-1)
    spec = prob["spec"]
    g0 = 1.0 + 0.01 * np.random.default_rng(7).standard_normal((spec.nseg, spec.ndet))
    want, _, _ = s.fit_gains(a1, tod, g0, per_detector=per_detector)  # [nseg][ndet]
    sums = tile_sums(s, a1, tod)
    got = sg.gains_from_sums(*sums, g0.T, per_detector=per_detector)  # [ndet][nseg]
    np.testing.assert_allclose(got.T, want, rtol=1e-12)


def test_operator_with_gains_is_the_tile_sum():
    """the oracle's operator with gains (every tile a one-segment detector
    with weights g^2 spn) equals sum_t P_t^T g_t^2 N_d^-1 P_t written out
    tile by tile from the oracle's pieces; b likewise with g"""
    import ctypes
    spec = synth.ProblemSpec("t", ndet=2, nside=8, nseg=3, ns=512, fknee=0.05, alpha=1.0,
                             problem=9)
    prob = synth.make_problem(spec)
    s = oracle.Setup(prob)
    L = oracle.lib()
    rng = np.random.default_rng(3)
    g = 1.0 + 0.1 * rng.standard_normal((spec.nseg, spec.ndet))  # [seg][det]
    x = rng.standard_normal(3 * s.npix)
    tod = np.ascontiguousarray(prob["tod"], np.float64).reshape(-1)
    ns = spec.ns
    want_a = np.zeros(3 * s.npix)
    want_b = np.zeros(3 * s.npix)
    for d in range(spec.ndet):
        for sg_ in range(spec.nseg):
            off = ns * sg_ + ns * spec.nseg * d
            pix = np.ascontiguousarray(s.pix[off:off + ns])
            psip = np.ascontiguousarray(s.psip[off:off + ns])
            pv = np.empty(ns)
            L.orc_deproject(oracle._pd(x), oracle._pl(s.indpix), oracle._pl(pix),
                            oracle._pd(psip), ctypes.c_long(ns), ctypes.c_long(s.npix),
                            oracle._pd(pv))
            gt = g[sg_, d]
            ya = gt * gt * s.noise_filter(d, pv)
            yb = gt * s.noise_filter(d, np.ascontiguousarray(tod[off:off + ns]))
            for y, acc in ((ya, want_a), (yb, want_b)):
                y = np.ascontiguousarray(y)
                L.orc_backproject(oracle._pd(acc), oracle._pl(s.indpix), oracle._pl(pix),
                                  oracle._pd(psip), ctypes.c_long(ns), ctypes.c_long(s.npix),
                                  oracle._pd(y))
    np.testing.assert_allclose(s.apply_gains(x, g), want_a, rtol=1e-12,
                               atol=1e-12 * np.abs(want_a).max())
    np.testing.assert_allclose(s.rhs_gains(tod, g), want_b, rtol=1e-12,
                               atol=1e-12 * np.abs(want_b).max())
    # gains 1: the operator without gains
    ones = np.ones_like(g)
    np.testing.assert_allclose(s.apply_gains(x, ones), s.apply(x), rtol=1e-12,
                               atol=1e-12 * np.abs(want_a).max())


def test_gain_arithmetic_edge_cases():
    """a tile without signal keeps its gain; no positive mean is an error"""
    import sanepic_gb300 as sg
    nd, nsg = 2, 3
    z2 = np.zeros((nd, nsg, 2))
    spn = np.zeros((nd, 2))
    g0 = np.full((nd, nsg), 1.2)
    bd = np.full((nd, nsg), 2.0)
    cs = np.full((nd, nsg), 1.0)
    cs[1, 2] = 0.0  # no signal in this tile
    got = sg.gains_from_sums(bd, cs, z2, z2, spn, g0)
    # raw gains 2 (and the old 1.2 where c = 0), scaled to mean 1.2
    raw = np.full((nd, nsg), 2.0)
    raw[1, 2] = 1.2
    np.testing.assert_allclose(got, raw * (1.2 / raw.mean()), rtol=1e-15)
    # -R sums a detector's segments
    got_d = sg.gains_from_sums(bd, cs, z2, z2, spn, g0, per_detector=True)
    assert np.ptp(got_d, axis=1).max() == 0.0
    with pytest.raises(sg.SanepicError):
        sg.gains_from_sums(-bd, cs, z2, z2, spn, g0)
