"""CPU oracle for the map-making hot path (TEST INFRASTRUCTURE ONLY).

Python bindings over liboracle.so, the FP64 restatement of the reference
(patanch/SANEPIC src/sanepic.cc, cited per function in oracle.h), plus a
driver that runs the reference's whole hot path on an in-memory problem.
Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use
this package; the GPU library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_d = ctypes.POINTER(ctypes.c_double)
_l = ctypes.POINTER(ctypes.c_long)


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, with ref=True, the shimmed reference)."""
    targets = ["oracle"] + (["ref"] if ref else [])
    subprocess.check_call(["make", "-s", "-C", HERE] + targets)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _LIB = ctypes.CDLL(path)
        _LIB.orc_ang2pix_ring.restype = ctypes.c_long
        _LIB.orc_indpix.restype = ctypes.c_long
        _LIB.orc_rhs.restype = ctypes.c_double
        _LIB.orc_gain_chi2.restype = ctypes.c_double
        _LIB.orc_pcg.restype = ctypes.c_int
        _LIB.orc_expand_detector.restype = ctypes.c_int
        _LIB.cp_run.restype = ctypes.c_int
    return _LIB


def _pd(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_d)


def _pl(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_l)


def ang2pix_ring(nside, theta, phi):
    L = lib()
    return np.array([L.orc_ang2pix_ring(ctypes.c_long(nside), ctypes.c_double(t),
                                        ctypes.c_double(p))
                     for t, p in zip(np.ravel(theta), np.ravel(phi))], np.int64)


class Setup:
    """Pixels, angles, indpix and noise weights for an in-memory problem."""

    def __init__(self, prob, det_offsets=None):
        L = lib()
        spec = prob["spec"]
        self.spec = spec
        ns, nseg, ndet, nside = spec.ns, spec.nseg, spec.ndet, spec.nside
        self.ns, self.nseg, self.ndet, self.nside = ns, nseg, ndet, nside
        nsd = ns * nseg
        self.pix = np.empty(ndet * nsd, np.int64)
        self.psip = np.empty(ndet * nsd)
        self.psipfp = np.empty(ndet * nsd)
        prev = ctypes.c_long(0)
        ra = np.ascontiguousarray(prob["ra"], np.float64)
        dec = np.ascontiguousarray(prob["dec"], np.float64)
        psi = np.ascontiguousarray(prob["psi"], np.float64)
        isamp = np.ascontiguousarray(prob["isampmin"], np.int64)
        for d in range(ndet):
            offx, offy = (0.0, 0.0) if det_offsets is None else det_offsets[d]
            psidet = prob["angles"][d] / 180.0 * 6.2831853071795864769252867665590057683943387987502 / 2.0
            sl = slice(d * nsd, (d + 1) * nsd)
            rc = L.orc_expand_detector(
                ctypes.c_long(ns), ctypes.c_long(nseg), _pl(isamp), _pd(ra), _pd(dec),
                _pd(psi), ctypes.c_double(offx), ctypes.c_double(offy),
                ctypes.c_double(psidet), ctypes.c_int(int(spec.hwp)),
                ctypes.c_double(prob["omega"]), ctypes.c_long(nside),
                _pl(self.pix[sl]), _pd(self.psip[sl]), _pd(self.psipfp[sl]),
                ctypes.byref(prev))
            if rc != 0:
                raise ValueError("ang2pix range error (the reference exits here)")
        self.indpix = np.empty(12 * nside * nside, np.int64)
        self.npix = L.orc_indpix(ctypes.c_long(nside), ctypes.c_long(self.pix.size),
                                 _pl(self.pix), _pl(self.indpix))
        self.spn = np.empty(ndet * ns)
        for d in range(ndet):
            ispf = np.ascontiguousarray(prob["ispf"][d], np.float64)
            L.orc_noise_weights(ctypes.c_long(ns), ctypes.c_long(ispf.size), _pd(ispf),
                                _pd(self.spn[d * ns:(d + 1) * ns]))
        self.hits = np.empty(2 * self.npix, np.int64)
        L.orc_hits(ctypes.c_long(self.pix.size), ctypes.c_long(self.npix),
                   _pl(self.indpix), _pl(self.pix), _pl(self.hits))

    # ---- operator pieces ------------------------------------------------
    def apply(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(3 * self.npix)
        lib().orc_apply(ctypes.c_long(self.ns), ctypes.c_long(self.nseg),
                        ctypes.c_long(self.ndet), ctypes.c_long(self.npix),
                        _pl(self.indpix), _pl(self.pix), _pd(self.psip), _pd(self.spn),
                        _pd(x), _pd(y))
        return y

    def rhs(self, tod):
        tod = np.ascontiguousarray(tod, np.float64).reshape(-1)
        b = np.empty(3 * self.npix)
        chi2 = lib().orc_rhs(ctypes.c_long(self.ns), ctypes.c_long(self.nseg),
                             ctypes.c_long(self.ndet), ctypes.c_long(self.npix),
                             _pl(self.indpix), _pl(self.pix), _pd(self.psip),
                             _pd(self.spn), _pd(tod), _pd(b))
        return b, chi2

    def noise_filter(self, det, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(self.ns)
        lib().orc_noise_filter(ctypes.c_long(self.ns), _pd(x),
                               _pd(self.spn[det * self.ns:(det + 1) * self.ns]), _pd(y))
        return y

    def sumcross(self):
        out = np.empty(3 * self.npix)
        lib().orc_sumcross(ctypes.c_long(self.pix.size), ctypes.c_long(self.npix),
                           _pl(self.indpix), _pl(self.pix), _pd(self.psipfp), _pd(out))
        return out

    def diag_precond(self):
        Mp = np.empty(3 * self.npix)
        lib().orc_diag_precond(ctypes.c_long(self.ns), ctypes.c_long(self.nseg),
                               ctypes.c_long(self.ndet), ctypes.c_long(self.npix),
                               _pl(self.indpix), _pl(self.pix), _pd(self.spn), _pd(Mp))
        return Mp

    def block_jacobi(self):
        minv = np.empty(9 * self.npix)
        lib().orc_block_jacobi(ctypes.c_long(self.ns), ctypes.c_long(self.nseg),
                               ctypes.c_long(self.ndet), ctypes.c_long(self.npix),
                               _pl(self.indpix), _pl(self.pix), _pd(self.psip),
                               _pd(self.spn), _pl(self.hits), _pd(minv))
        return minv

    def pcg(self, b, precond="diag", x0=None, stop_crit=1e-15, maxiter=2000,
            verbose=False, Mp=None, minv=None):
        n = 3 * self.npix
        x = np.empty(n)
        hist = np.zeros(maxiter + 1)
        pc = {"diag": 0, "bj3": 1}[precond]
        if pc == 0 and Mp is None:
            Mp = self.diag_precond()
        if pc == 1 and minv is None:
            minv = self.block_jacobi()
        Mp_arr = np.ascontiguousarray(Mp if Mp is not None else np.zeros(n))
        minv_arr = np.ascontiguousarray(minv if minv is not None else np.zeros(9 * self.npix))
        x0p = _pd(np.ascontiguousarray(x0, np.float64)) if x0 is not None else None
        it = lib().orc_pcg(ctypes.c_long(self.ns), ctypes.c_long(self.nseg),
                           ctypes.c_long(self.ndet), ctypes.c_long(self.npix),
                           _pl(self.indpix), _pl(self.pix), _pd(self.psip), _pd(self.spn),
                           _pd(np.ascontiguousarray(b, np.float64)), _pl(self.hits),
                           _pd(Mp_arr), _pd(minv_arr), ctypes.c_int(pc), x0p,
                           ctypes.c_double(stop_crit), ctypes.c_int(maxiter),
                           ctypes.c_int(int(verbose)), _pd(x), _pd(hist))
        return x, it, hist[:it]

    # ---- recalibration: per-tile gains (sanepic.cc:1041-1130, 2123-2316) --
    # A tile (det, seg) is its own one-segment "detector": the [det][seg]
    # sample layout is already [tile][sample], so the operator with gains is
    # orc_apply / orc_rhs / orc_pcg over ndet * nseg one-segment detectors,
    # each with its detector's weights times g^2 (A) or g (b = P^T G N^-1 d).
    def _tile_spn(self, scale):
        """spn of every tile [det][seg] times scale[det][seg]."""
        sc = np.asarray(scale, np.float64).reshape(self.ndet, self.nseg, 1)
        return np.ascontiguousarray((self.spn.reshape(self.ndet, 1, self.ns) * sc).reshape(-1))

    def _gains_ds(self, gains):
        """gains in the reference's [seg][det] layout -> [det][seg]."""
        return np.ascontiguousarray(np.asarray(gains, np.float64).reshape(self.nseg, self.ndet).T)

    def apply_gains(self, x, gains):
        g = self._gains_ds(gains)
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(3 * self.npix)
        lib().orc_apply(ctypes.c_long(self.ns), ctypes.c_long(1),
                        ctypes.c_long(self.ndet * self.nseg), ctypes.c_long(self.npix),
                        _pl(self.indpix), _pl(self.pix), _pd(self.psip),
                        _pd(self._tile_spn(g * g)), _pd(x), _pd(y))
        return y

    def rhs_gains(self, tod, gains):
        g = self._gains_ds(gains)
        tod = np.ascontiguousarray(tod, np.float64).reshape(-1)
        b = np.empty(3 * self.npix)
        lib().orc_rhs(ctypes.c_long(self.ns), ctypes.c_long(1),
                      ctypes.c_long(self.ndet * self.nseg), ctypes.c_long(self.npix),
                      _pl(self.indpix), _pl(self.pix), _pd(self.psip), _pd(self._tile_spn(g)),
                      _pd(tod), _pd(b))
        return b

    def pcg_gains(self, b, gains, precond="diag", x0=None, stop_crit=1e-15, maxiter=2000,
                  Mp=None, minv=None):
        """PCG on P^T G N^-1 G P with the preconditioner made without gains
        (the reference keeps that of its first loop, sanepic.cc:1352)."""
        g = self._gains_ds(gains)
        n = 3 * self.npix
        x = np.empty(n)
        hist = np.zeros(maxiter + 1)
        pc = {"diag": 0, "bj3": 1}[precond]
        if pc == 0 and Mp is None:
            Mp = self.diag_precond()
        if pc == 1 and minv is None:
            minv = self.block_jacobi()
        Mp_arr = np.ascontiguousarray(Mp if Mp is not None else np.zeros(n))
        minv_arr = np.ascontiguousarray(minv if minv is not None else np.zeros(9 * self.npix))
        x0p = _pd(np.ascontiguousarray(x0, np.float64)) if x0 is not None else None
        it = lib().orc_pcg(ctypes.c_long(self.ns), ctypes.c_long(1),
                           ctypes.c_long(self.ndet * self.nseg), ctypes.c_long(self.npix),
                           _pl(self.indpix), _pl(self.pix), _pd(self.psip),
                           _pd(self._tile_spn(g * g)),
                           _pd(np.ascontiguousarray(b, np.float64)), _pl(self.hits),
                           _pd(Mp_arr), _pd(minv_arr), ctypes.c_int(pc), x0p,
                           ctypes.c_double(stop_crit), ctypes.c_int(maxiter), ctypes.c_int(0),
                           _pd(x), _pd(hist))
        return x, it, hist[:it]

    def gain_dots(self, x, tod):
        """(b, c) per tile [det][seg]: 2 sum_k Re(D conj S) spn and
        2 sum_k |S|^2 spn over the half spectrum, S = r2c(P x), D = r2c(d)."""
        tod = np.ascontiguousarray(tod, np.float64).reshape(-1)
        nt = self.ndet * self.nseg
        dots = np.empty(2 * nt)
        lib().orc_gain_dots(ctypes.c_long(self.ns), ctypes.c_long(self.nseg),
                            ctypes.c_long(self.ndet), ctypes.c_long(self.npix),
                            _pl(self.indpix), _pl(self.pix), _pd(self.psip), _pd(self.spn),
                            _pd(tod), _pd(np.ascontiguousarray(x, np.float64)), _pd(dots))
        return (dots[:nt].reshape(self.ndet, self.nseg), dots[nt:].reshape(self.ndet, self.nseg))

    def gain_chi2(self, x, tod, gains=None):
        tod = np.ascontiguousarray(tod, np.float64).reshape(-1)
        gp = _pd(self._gains_ds(gains)) if gains is not None else None
        return lib().orc_gain_chi2(ctypes.c_long(self.ns), ctypes.c_long(self.nseg),
                                   ctypes.c_long(self.ndet), ctypes.c_long(self.npix),
                                   _pl(self.indpix), _pl(self.pix), _pd(self.psip),
                                   _pd(self.spn), _pd(tod),
                                   _pd(np.ascontiguousarray(x, np.float64)), gp)

    def fit_gains(self, x, tod, gains_old, per_detector=False):
        """The recalibration fit with the map x fixed (sanepic.cc:2166-2291):
        g = b / c per tile (per detector with -R: sums over its segments),
        then scaled so that the mean gain equals that of gains_old.  Returns
        (gains [nseg][ndet], chi2 before, chi2 after)."""
        bd, cs = self.gain_dots(x, tod)
        g0 = self._gains_ds(gains_old)
        if per_detector:
            zeta, gamma = bd.sum(axis=1, keepdims=True), cs.sum(axis=1, keepdims=True)
            g = np.where(gamma > 0, zeta / np.where(gamma > 0, gamma, 1.0), g0)
            g = np.broadcast_to(g, g0.shape).copy()
        else:
            g = np.where(cs > 0, bd / np.where(cs > 0, cs, 1.0), g0)
        g *= g0.sum() / g.sum()
        gr = np.ascontiguousarray(g.T)
        return gr, self.gain_chi2(x, tod, gains_old), self.gain_chi2(x, tod, gr)

    def expand(self, compact):
        compact = np.ascontiguousarray(compact, np.float64)
        full = np.empty(12 * self.nside * self.nside)
        lib().orc_expand_map(ctypes.c_long(self.nside), _pl(self.indpix), _pd(compact),
                             _pd(full))
        return full


def masked(setup: Setup) -> np.ndarray:
    """Boolean [3*npix]: Q/U entries the reference zeroes (pol hits < 4)."""
    m = np.zeros(3 * setup.npix, bool)
    pol = setup.hits[setup.npix:] < 4
    m[setup.npix:2 * setup.npix] = pol
    m[2 * setup.npix:] = pol
    return m


def run_pipeline(prob, precond="diag", stop_crit=1e-15, maxiter=2000, verbose=False):
    """The reference's whole hot path on one problem; returns its outputs as a
    dict of full RING maps (plus 'A', the compact solution) and metadata."""
    s = Setup(prob)
    tod = np.ascontiguousarray(prob["tod"], np.float64).reshape(-1)
    b, chi20 = s.rhs(tod)
    Mp = s.diag_precond()
    x, iters, hist = s.pcg(b, precond=precond, stop_crit=stop_crit, maxiter=maxiter,
                           verbose=verbose, Mp=Mp)
    npix = s.npix
    msk = masked(s)
    Mpm = Mp.copy()
    Mpm[msk] = 0.0
    nvar = np.where(Mpm != 0.0, 1.0 / np.where(Mpm != 0.0, Mpm, 1.0), 0.0)
    sc = s.sumcross()
    sc[msk] = 0.0
    out = {
        "A": x, "I": s.expand(x[:npix]), "Q": s.expand(x[npix:2 * npix]),
        "U": s.expand(x[2 * npix:]), "NVAR": s.expand(nvar[:npix]),
        "Q_NVAR": s.expand(nvar[npix:2 * npix]), "U_NVAR": s.expand(nvar[2 * npix:]),
        "HITS": s.expand(s.hits[:npix].astype(np.float64)),
        "POL_HITS": s.expand(s.hits[npix:].astype(np.float64)),
        "COS2P": s.expand(sc[:npix]), "SIN2P": s.expand(sc[npix:2 * npix]),
    }
    return out, dict(iters=iters, crit=hist, chi20=chi20, npix=npix, setup=s)


def cpu_solve(prob, nthreads: int, stop_crit: float = 1e-12, maxiter: int = 2000):
    """The reference's whole path (setup, RHS, diagonal preconditioner, PCG)
    on nthreads host threads in its parallel layout (cgpar.c).  Returns the
    compact solution, the iteration count, crit per iteration and the phase
    times (seconds): setup, rhs, precond, solve, and to_stop = from the end of
    setup until crit first reached stop_crit (-1 if it never did)."""
    L = lib()
    spec = prob["spec"]
    ns, nseg, ndet, nside = spec.ns, spec.nseg, spec.ndet, spec.nside
    ra = np.ascontiguousarray(prob["ra"], np.float64)
    dec = np.ascontiguousarray(prob["dec"], np.float64)
    psi = np.ascontiguousarray(prob["psi"], np.float64)
    isamp = np.ascontiguousarray(prob["isampmin"], np.int64)
    psidet = np.ascontiguousarray(np.asarray(prob["angles"], np.float64) / 180.0
                                  * 6.2831853071795864769252867665590057683943387987502 / 2.0)
    ispf = np.ascontiguousarray(prob["ispf"], np.float64)
    tod = np.ascontiguousarray(prob["tod"], np.float64)
    x = np.zeros(3 * 12 * nside * nside)
    hist = np.zeros(maxiter + 1)
    times = np.zeros(5)
    npix = ctypes.c_long(0)
    iters = ctypes.c_int(0)
    rc = L.cp_run(ctypes.c_long(ns), ctypes.c_long(nseg), ctypes.c_long(ndet),
                  ctypes.c_long(nside), _pd(ra), _pd(dec), _pd(psi), _pl(isamp), _pd(psidet),
                  ctypes.c_int(int(spec.hwp)), ctypes.c_double(prob["omega"]), _pd(ispf),
                  ctypes.c_long(ispf.shape[1]), _pd(tod), ctypes.c_int(nthreads),
                  ctypes.c_double(stop_crit), ctypes.c_int(maxiter), _pd(x), _pd(hist),
                  _pd(times), ctypes.byref(npix), ctypes.byref(iters))
    if rc != 0:
        raise ValueError(f"cp_run failed ({rc})")
    n = npix.value
    it = iters.value
    return {"x": x[:3 * n].copy(), "npix": n, "iterations": it, "crit": hist[:it].copy(),
            "times": dict(zip(("setup", "rhs", "precond", "solve", "to_stop"), times.tolist()))}
