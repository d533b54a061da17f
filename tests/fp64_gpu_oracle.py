"""An FP64 GPU operator for map-making, written independently of the library
(TEST INFRASTRUCTURE ONLY): plain torch float64 arithmetic, cuFFT through
torch.fft, and index_add_ for P^T.  It restates the reference's operator
(patanch/SANEPIC src/sanepic.cc):

  P      deproject, sanepic.cc:2845-2873: y = I[m] + cos 2psi Q[m] + sin 2psi U[m]
  N^-1   do_PtNd, sanepic.cc:2522-2582 with the weights of 507-539: FFTW r2c,
         x SpN[k] = iSpf[k ns_sp / ns] / ns^2 (bin 0: iSpf[1] 1e-6 / ns^2),
         unnormalised c2r
  P^T    sanepic.cc:2584-2611, Q/U zeroed where the pol mask applies
         (fewer than 2 true hits, sanepic.cc:1316-1330, 1455-1459)

and solves A m = b with its own conjugate gradient in FP64.  It shares no
code with the library: it catches mistakes that the library's own FP64 mode
would repeat.  Pixels and angles come from the CPU oracle (the reference's
pointing expansion and ang2pix, bit-exact with it).  It serves problems whose
detectors all sit on the boresight (every C2/C3-style configuration), where
one pointing expansion gives every detector's pixels.
"""
from __future__ import annotations

import math

import numpy as np

D2PI = 6.2831853071795864769252867665590057683943387987502


class Fp64Operator:
    def __init__(self, prob, device="cuda"):
        import torch

        import oracle

        self.torch = torch
        spec = prob["spec"]
        self.spec = spec
        self.dev = device
        ns, nseg, ndet = spec.ns, spec.nseg, spec.ndet
        self.ns, self.nseg, self.ndet = ns, nseg, ndet
        # one pointing expansion with a zero detector angle: its psi is the
        # boresight angle after pointingshift; detector d adds its own angle
        # (sanepic.cc:757-766)
        one = dict(prob)
        one["spec"] = _replace(spec, ndet=1)
        one["angles"] = np.zeros(1)
        s = oracle.Setup(one)
        self.npix = s.npix
        self.indpix = s.indpix
        m = s.indpix[s.pix]
        assert (m >= 0).all()
        self.m = torch.tensor(m, dtype=torch.int64, device=device)
        # psipfp: the angle without the half-wave plate term (sanepic.cc:760-762)
        self.psi0 = torch.tensor(s.psipfp, dtype=torch.float64, device=device)
        self.psidet = [float(a) / 180.0 * D2PI / 2.0 for a in prob["angles"]]
        self.hwp = bool(spec.hwp)
        if self.hwp:
            # absolute sample index ii + ns * iseg (sanepic.cc:765)
            t = torch.arange(ns * nseg, dtype=torch.float64, device=device)
            self.hwp_term = 2.0 * float(prob["omega"]) * t
        # noise weights per detector (sanepic.cc:533-537), rFFT bins k = 0..ns/2
        self.spn = []
        k = np.arange(ns // 2 + 1, dtype=np.float64)
        for d in range(ndet):
            ispf = prob["ispf"][d]
            w = ispf[(k * ispf.size / ns).astype(np.int64)] / ns / ns
            w[0] = ispf[1] * 1e-6 / ns / ns
            self.spn.append(torch.tensor(w, dtype=torch.float64, device=device))
        # hits per observed pixel (true counts, every detector) and the pol mask
        self.hits = torch.bincount(self.m, minlength=self.npix).to(torch.float64) * ndet
        self.pol = (self.hits >= 2).to(torch.float64)

    def angles(self, d):
        """(cos 2psi, sin 2psi) of detector d, FP64 on the device."""
        torch = self.torch
        p = self.psi0 + self.psidet[d]
        if self.hwp:
            p = -p + self.hwp_term
        return torch.cos(2.0 * p), torch.sin(2.0 * p)

    def noise(self, d, y):
        """N_d^-1 applied segment by segment: c2r(r2c(y) SpN), FFTW scaling."""
        torch = self.torch
        Y = torch.fft.rfft(y.view(self.nseg, self.ns), dim=1) * self.spn[d]
        return (torch.fft.irfft(Y, n=self.ns, dim=1) * self.ns).reshape(-1)

    def pt(self, acc, d, yw, c, s):
        acc[0].index_add_(0, self.m, yw)
        acc[1].index_add_(0, self.m, c * yw)
        acc[2].index_add_(0, self.m, s * yw)

    def _masked(self, acc):
        acc[1] *= self.pol
        acc[2] *= self.pol
        return acc.reshape(-1)

    def apply(self, x):
        """A x = P^T N^-1 P x, masked (x: [3 npix] FP64 on the device)."""
        torch = self.torch
        xv = x.view(3, self.npix)
        acc = torch.zeros(3, self.npix, dtype=torch.float64, device=self.dev)
        for d in range(self.ndet):
            c, s = self.angles(d)
            y = xv[0][self.m] + c * xv[1][self.m] + s * xv[2][self.m]
            self.pt(acc, d, self.noise(d, y), c, s)
        return self._masked(acc)

    def rhs(self, tod):
        """b = P^T N^-1 d (tod: host [ndet][nseg*ns] FP64)."""
        torch = self.torch
        acc = torch.zeros(3, self.npix, dtype=torch.float64, device=self.dev)
        for d in range(self.ndet):
            c, s = self.angles(d)
            y = torch.tensor(np.ascontiguousarray(tod[d], np.float64), device=self.dev)
            self.pt(acc, d, self.noise(d, y), c, s)
        return self._masked(acc)

    def block_jacobi(self):
        """Inverses of the per-pixel 3x3 blocks of unit-weight hits (any SPD
        preconditioner gives the same converged map)."""
        torch = self.torch
        W = torch.zeros(self.npix, 3, 3, dtype=torch.float64, device=self.dev)
        for d in range(self.ndet):
            c, s = self.angles(d)
            w = torch.stack([torch.ones_like(c), c, s], 1)
            for i in range(3):
                for j in range(3):
                    W[:, i, j].index_add_(0, self.m, w[:, i] * w[:, j])
        pol = self.pol.bool()
        W[~pol, 1:, :] = 0.0
        W[~pol, :, 1:] = 0.0
        W[~pol, 1, 1] = 1.0
        W[~pol, 2, 2] = 1.0
        inv = torch.linalg.inv(W)
        inv[~pol, 1:, :] = 0.0
        inv[~pol, :, 1:] = 0.0
        return inv

    def solve(self, b, stop=1e-22, maxiter=500):
        """PCG in FP64 to |r|^2/|b|^2 <= stop; returns (x, iterations, crit)."""
        torch = self.torch
        Minv = self.block_jacobi()

        def M(r):
            return torch.einsum("pij,jp->ip", Minv, r.view(3, self.npix)).reshape(-1)

        x = torch.zeros_like(b)
        r = b.clone()
        z = M(r)
        d = z.clone()
        rz = torch.dot(r, z)
        bb = torch.dot(b, b)
        it, crit = 0, 1.0
        while it < maxiter:
            q = self.apply(d)
            alpha = rz / torch.dot(d, q)
            x += alpha * d
            if it % 10 == 9:
                r = b - self.apply(x)
            else:
                r -= alpha * q
            z = M(r)
            rz_new = torch.dot(r, z)
            d = z + (rz_new / rz) * d
            rz = rz_new
            it += 1
            crit = float(torch.dot(r, r) / bb)
            if crit <= stop:
                break
        return x, it, crit

    def compact_to_ring_order(self, x):
        """The solution in the reference's compact order (observed pixels in
        ascending RING) as host [3][npix]."""
        return x.view(3, self.npix).cpu().numpy()


def _replace(spec, **kw):
    import dataclasses
    return dataclasses.replace(spec, **kw)


def map_errors(got, want, monopole=False):
    """Max and RMS error of `got` relative to `want` (max |want|, RMS of
    want); with monopole=True the mean difference is removed first."""
    d = np.asarray(got, np.float64) - np.asarray(want, np.float64)
    if monopole:
        d = d - d.mean()
    scale_rms = math.sqrt(float(np.mean(np.square(want))))
    scale_max = float(np.max(np.abs(want)))
    return {"rms": math.sqrt(float(np.mean(np.square(d)))) / scale_rms,
            "max": float(np.max(np.abs(d))) / scale_max}
