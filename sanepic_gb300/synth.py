"""Seeded synthetic map-making problems in the reference's input formats.

The reference ships no data set (its README points at litebird_sim output,
which is not available here), so every problem is generated:

* Scan: the spin axis sits 45 deg from an anti-sun axis that advances one turn
  per year and precesses about it with a 3 h period; the boresight sits 50 deg
  from the spin axis and spins with a 60 s period; fsamp = 19 Hz; the timeline
  is contiguous with segment i = samples [i*ns, (i+1)*ns - 1].  psi is the
  angle of the scan direction relative to the local meridian.  Stored as the
  reference expects (README.md:58-64): dec in (-pi/2, pi/2], ra in [0, 2pi).
* Sky: iid per RING pixel, I ~ N(0, (100 uK)^2), Q, U ~ N(0, (10 uK)^2), in K.
* TOD: I + Q cos 2psi' + U sin 2psi' + n, psi' being the reference's psip
  (sanepic.cc:757-766, HWP included), n Gaussian with per-segment circulant
  PSD  sigma^2 (1 + (f/fknee)^-alpha),  sigma = 50 uK sqrt(s) sqrt(fsamp).
* iSpf[k] = 1 / PSD(f_min(k, ns-k)) for k < ns (bin 0 uses bin 1; the
  reference overwrites it anyway, sanepic.cc:536-537).
* Seeds: sky 1000+problem, noise 2000+1000*problem+det, detector draws
  3000+problem.

`write_reference_tree` lays the files out exactly as scripts/run_sanepic.sh
expects and returns the matching command-line arguments.
"""
from __future__ import annotations

import concurrent.futures
import dataclasses
import math
import os
from typing import Dict, List, Optional

import numpy as np

D2PI = 6.2831853071795864769252867665590057683943387987502
FSAMP = 19.0


@dataclasses.dataclass
class ProblemSpec:
    name: str
    ndet: int
    nside: int
    nseg: int
    ns: int
    hwp: bool = False
    fknee: float = 0.1          # Hz, used when fknee_range is None
    alpha: float = 1.0
    fknee_range: Optional[tuple] = None   # per-detector U[a, b]
    alpha_range: Optional[tuple] = None
    sigma_uk: float = 50.0
    problem: int = 0            # seed offset
    precision: str = "f64"      # operator precision: "f64" or "f32"
    noise: bool = True
    angle_mode: str = "uniform"  # detector orientations


# Configurations named after the workloads they describe.
PRESETS: Dict[str, ProblemSpec] = {
    # 1 detector, NSIDE 64, 12 x 65,536 samples, FP64
    "c1_1det_nside64": ProblemSpec("c1_1det_nside64", 1, 64, 12, 65536,
                                   fknee=0.1, alpha=1.0, precision="f64"),
    # the same scan and sizes with 4 detectors at seeded orientations (well
    # posed: one detector angle leaves most Q/U blocks nearly singular)
    "c1_4det_nside64": ProblemSpec("c1_4det_nside64", 4, 64, 12, 65536,
                                   fknee=0.1, alpha=1.0, problem=3, precision="f64"),
    # 64 detectors, NSIDE 256, 48 x 131,072 samples, per-detector 1/f, FP32
    "c2_64det_nside256": ProblemSpec("c2_64det_nside256", 64, 256, 48, 131072,
                                     fknee_range=(0.02, 0.2),
                                     alpha_range=(1.0, 2.0), precision="f32"),
    # the same tiles with 8 detectors: a small case for profiling captures
    "c2_8det_nside256": ProblemSpec("c2_8det_nside256", 8, 256, 48, 131072,
                                    fknee_range=(0.02, 0.2),
                                    alpha_range=(1.0, 2.0), precision="f32"),
    # 256 detectors, NSIDE 512, 48 x 131,072 samples, HWP, FP32
    "c3_256det_nside512_hwp": ProblemSpec("c3_256det_nside512_hwp", 256, 512,
                                          48, 131072, hwp=True, fknee=0.05,
                                          alpha=1.5, precision="f32"),
}


def spec_from_name(name: str) -> ProblemSpec:
    return dataclasses.replace(PRESETS[name])


def batch_specs(n: int = 32, seed: int = 500) -> List[ProblemSpec]:
    """Uneven independent problems for batched solves: detector counts from
    {1, 4, 16, 64}, NSIDE from {64, 128, 256}, segment lengths from {16384,
    65536, 131072} with 8-48 segments, f_knee ~ U[0.02, 0.2] Hz (one per
    problem), FP32 operator.  Seeded: the same list every call."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        ndet = int(rng.choice([1, 4, 16, 64]))
        nside = int(rng.choice([64, 128, 256]))
        ns = int(rng.choice([16384, 65536, 131072]))
        nseg = int(rng.integers(8, 49))
        fk = float(rng.uniform(0.02, 0.2))
        out.append(ProblemSpec(f"batch{i:02d}_{ndet}det_nside{nside}_{nseg}x{ns}", ndet, nside,
                               nseg, ns, fknee=fk, alpha=1.0, problem=seed + i,
                               precision="f32"))
    return out


# --------------------------------------------------------------------------
# HEALPix RING ang2pix, vectorised FP64 restatement of the reference's
# ang2pix_ring (sanepic.cc:2764-2843); used only to paint the sky into TODs.
def ang2pix_ring(nside: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    theta = np.asarray(theta, np.float64)
    phi = np.asarray(phi, np.float64).copy()
    z = np.cos(theta)
    za = np.abs(z)
    phi = np.where(phi >= 2.0 * math.pi, phi - 2.0 * math.pi, phi)
    phi = np.where(phi < 0.0, phi + 2.0 * math.pi, phi)
    tt = phi / (0.5 * math.pi)
    nl4 = 4 * nside
    ncap = 2 * nside * (nside - 1)
    npix = 12 * nside * nside
    out = np.empty(theta.shape, np.int64)
    eq = za <= 2.0 / 3.0
    # equatorial belt
    t, zz = tt[eq], z[eq]
    jp = np.floor(nside * (0.5 + t - zz * 0.75)).astype(np.int64)
    jm = np.floor(nside * (0.5 + t + zz * 0.75)).astype(np.int64)
    ir = nside + 1 + jp - jm
    kshift = 1 - (ir & 1)
    num = jp + jm - nside + kshift + 1
    ip = np.trunc(num / 2).astype(np.int64) + 1   # C integer division
    ip = np.where(ip > nl4, ip - nl4, ip)
    out[eq] = ncap + nl4 * (ir - 1) + ip - 1
    # polar caps
    pc = ~eq
    t, zz, zab = tt[pc], z[pc], za[pc]
    tp = t - np.floor(t)
    tmp = np.sqrt(3.0 * (1.0 - zab))
    jp = np.floor(nside * tp * tmp).astype(np.int64)
    jm = np.floor(nside * (1.0 - tp) * tmp).astype(np.int64)
    ir = jp + jm + 1
    ip = np.floor(t * ir).astype(np.int64) + 1
    ip = np.where(ip > 4 * ir, ip - 4 * ir, ip)
    pix = 2 * ir * (ir - 1) + ip
    pix = np.where(zz <= 0.0, npix - 2 * ir * (ir + 1) + ip, pix)
    out[pc] = pix - 1
    return out


# --------------------------------------------------------------------------
def scan_pointing(nsamp: int, fsamp: float = FSAMP, t0: float = 0.0,
                  spin_period: float = 60.0, prec_period: float = 3 * 3600.0,
                  spin_axis_deg: float = 45.0, boresight_deg: float = 50.0):
    """Boresight (ra, dec, psi) in radians for a spin + precession scan."""
    t = t0 + np.arange(nsamp, dtype=np.float64) / fsamp
    lam = D2PI * t / (365.25 * 86400.0)
    a = np.stack([np.cos(lam), np.sin(lam), np.zeros_like(lam)])
    e1 = np.stack([np.zeros_like(lam), np.zeros_like(lam), np.ones_like(lam)])
    e2 = np.stack([np.sin(lam), -np.cos(lam), np.zeros_like(lam)])
    php = D2PI * t / prec_period
    ca, sa = math.cos(math.radians(spin_axis_deg)), math.sin(math.radians(spin_axis_deg))
    s = ca * a + sa * (np.cos(php) * e1 + np.sin(php) * e2)
    zhat = np.array([0.0, 0.0, 1.0])[:, None]
    u1 = zhat - (s[2][None, :]) * s
    u1 /= np.linalg.norm(u1, axis=0, keepdims=True)
    u2 = np.cross(s.T, u1.T).T
    phs = D2PI * t / spin_period
    cb, sb = math.cos(math.radians(boresight_deg)), math.sin(math.radians(boresight_deg))
    b = cb * s + sb * (np.cos(phs) * u1 + np.sin(phs) * u2)
    p = -np.sin(phs) * u1 + np.cos(phs) * u2
    dec = np.arcsin(np.clip(b[2], -1.0, 1.0))
    ra = np.mod(np.arctan2(b[1], b[0]), D2PI)
    north = np.stack([-np.sin(dec) * np.cos(ra), -np.sin(dec) * np.sin(ra), np.cos(dec)])
    east = np.stack([-np.sin(ra), np.cos(ra), np.zeros_like(ra)])
    psi = np.arctan2((p * east).sum(0), (p * north).sum(0))
    return ra, dec, psi


def detector_table(spec: ProblemSpec):
    """Detector names, orientation angles (deg) and noise parameters."""
    rng = np.random.default_rng(3000 + spec.problem)
    if spec.ndet == 1:
        angles = np.array([0.0])
    else:
        angles = rng.uniform(0.0, 180.0, spec.ndet)
    if spec.fknee_range:
        fk = rng.uniform(*spec.fknee_range, spec.ndet)
    else:
        fk = np.full(spec.ndet, spec.fknee)
    if spec.alpha_range:
        al = rng.uniform(*spec.alpha_range, spec.ndet)
    else:
        al = np.full(spec.ndet, spec.alpha)
    names = [f"DET{d:04d}" for d in range(spec.ndet)]
    return names, angles, fk, al


def psd(spec: ProblemSpec, fknee: float, alpha: float) -> np.ndarray:
    """PSD per rFFT bin k = 0..ns/2 (bin 0 takes bin 1's value)."""
    ns = spec.ns
    f = np.arange(ns // 2 + 1, dtype=np.float64) * FSAMP / ns
    f[0] = f[1]
    sigma = spec.sigma_uk * 1e-6 * math.sqrt(FSAMP)
    return sigma * sigma * (1.0 + (f / fknee) ** (-alpha))


def ispf_file_values(spec: ProblemSpec, fknee: float, alpha: float) -> np.ndarray:
    """iSpf values k = 0..ns-1 as the reference reads them (`-u` = ns)."""
    p = psd(spec, fknee, alpha)
    ns = spec.ns
    k = np.arange(ns)
    return 1.0 / p[np.minimum(k, ns - k)]


def make_sky(spec: ProblemSpec, seed: Optional[int] = None) -> np.ndarray:
    rng = np.random.default_rng(1000 + spec.problem if seed is None else seed)
    npix = 12 * spec.nside * spec.nside
    sky = np.empty((3, npix))
    sky[0] = rng.normal(0.0, 100e-6, npix)
    sky[1] = rng.normal(0.0, 10e-6, npix)
    sky[2] = rng.normal(0.0, 10e-6, npix)
    return sky


def hwp_omega() -> float:
    """HWP angular step in rad/sample: the TOD then carries 4*2pi*1.5 Hz."""
    return D2PI * 1.5 / FSAMP


def make_problem(spec: ProblemSpec, sky: Optional[np.ndarray] = None,
                 with_tod: bool = True, noise_seed_base: Optional[int] = None):
    """Everything in host memory: pointing, detectors, iSpf, TOD (FP64)."""
    nsamp = spec.nseg * spec.ns
    ra, dec, psi = scan_pointing(nsamp)
    names, angles, fk, al = detector_table(spec)
    if sky is None:
        sky = make_sky(spec)
    ispf = np.stack([ispf_file_values(spec, fk[d], al[d]) for d in range(spec.ndet)])
    prob = dict(spec=spec, ra=ra, dec=dec, psi=psi, names=names, angles=angles,
                fknee=fk, alpha=al, ispf=ispf, sky=sky,
                isampmin=np.arange(spec.nseg, dtype=np.int64) * spec.ns,
                omega=hwp_omega() if spec.hwp else 0.0)
    if with_tod:
        prob["tod"] = make_tod(prob, noise_seed_base=noise_seed_base)
    return prob


def make_tod(prob, noise_seed_base: Optional[int] = None, dets=None) -> np.ndarray:
    spec = prob["spec"]
    ns, nseg = spec.ns, spec.nseg
    nsamp = ns * nseg
    theta = D2PI / 4.0 - prob["dec"]
    phi = np.mod(prob["ra"] + D2PI, D2PI)
    pix = ang2pix_ring(spec.nside, theta, phi)
    sky = prob["sky"]
    I, Q, U = sky[0][pix], sky[1][pix], sky[2][pix]
    tidx = np.arange(nsamp, dtype=np.float64)
    dets = list(range(spec.ndet) if dets is None else dets)
    out = np.empty((len(dets), nsamp))
    base = 2000 + 1000 * spec.problem if noise_seed_base is None else noise_seed_base

    def one(j):
        d = dets[j]
        pdet = prob["psi"] + prob["angles"][d] / 180.0 * D2PI / 2.0
        if spec.hwp:
            pdet = -pdet + 2.0 * prob["omega"] * tidx
        tod = I + Q * np.cos(2.0 * pdet) + U * np.sin(2.0 * pdet)
        if spec.noise:
            rng = np.random.default_rng(base + d)
            amp = np.sqrt(psd(spec, prob["fknee"][d], prob["alpha"][d]))
            for g in range(nseg):
                w = rng.standard_normal(ns)
                n = np.fft.irfft(np.fft.rfft(w) * amp, n=ns)
                tod[g * ns:(g + 1) * ns] += n
        out[j] = tod

    # detectors are independent (own seed each): generate them on threads
    workers = min(len(dets), os.cpu_count() or 1)
    if workers > 1 and nsamp * len(dets) > 4_000_000:
        with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
            list(ex.map(one, range(len(dets))))
    else:
        for j in range(len(dets)):
            one(j)
    return out


# --------------------------------------------------------------------------
def write_reference_tree(prob, base_dir: str, ispf_prefix: str = "iSpf0.1_19.0_index1.0__"):
    """Write the reference's input files and return its argv (without argv[0]).

    Layout and flags follow scripts/run_sanepic.sh:8-73.
    """
    spec = prob["spec"]
    for sub in ("bolo_info", "out_dir", "pointings_list", "segments", "tod_list"):
        os.makedirs(os.path.join(base_dir, sub), exist_ok=True)
    bolofile = os.path.join(base_dir, "bolo_info", "bolometer_info.txt")
    with open(bolofile, "w") as f:
        for d, name in enumerate(prob["names"]):
            f.write(f"{d} {d} 0.0 0.0 {float(prob['angles'][d]):.17g} LFT {name}\n")
    detlist = os.path.join(base_dir, "bolo_info", "detector_list.txt")
    with open(detlist, "w") as f:
        for name in prob["names"]:
            f.write(name + "\n")
    for d, name in enumerate(prob["names"]):
        prob["ispf"][d].astype("<f8").tofile(
            os.path.join(base_dir, "bolo_info", ispf_prefix + name))
    pdir = os.path.join(base_dir, "pointings_list", "pointings_")
    prob["ra"].astype("<f8").tofile(pdir + "ra.bi")
    prob["dec"].astype("<f8").tofile(pdir + "dec.bi")
    prob["psi"].astype("<f8").tofile(pdir + "psi.bi")
    segfile = os.path.join(base_dir, "segments", f"segment_list_{spec.nseg}_{spec.ns}.bi")
    seg = np.empty(2 * spec.nseg, np.int64)
    seg[0::2] = np.arange(spec.nseg) * spec.ns
    seg[1::2] = (np.arange(spec.nseg) + 1) * spec.ns - 1
    seg.tofile(segfile)
    if "tod" in prob:
        for d, name in enumerate(prob["names"]):
            prob["tod"][d].astype("<f8").tofile(
                os.path.join(base_dir, "tod_list", f"data_{name}output.bi"))
    termin = f"output_N{spec.nside}_.bin"
    args = ["-F", os.path.join(base_dir, "tod_list") + "/", "-B", "output",
            "-f", segfile, "-d", str(spec.ndet)]
    if spec.ndet == 1:
        args += ["-C", prob["names"][0]]
    else:
        args += ["-D", detlist]
    args += ["-e", termin, "-h", "1" if spec.hwp else "0",
             "-w", repr(float(prob["omega"])) if spec.hwp else "1.123456789123",
             "-k", os.path.join(base_dir, "bolo_info", ispf_prefix),
             "-u", str(spec.ns), "-O", os.path.join(base_dir, "out_dir", "map_"),
             "-p", "1", "-l", str(spec.ns), "-n", str(spec.nseg),
             "-N", str(spec.nside), "-X", bolofile,
             "-Z", os.path.join(base_dir, "pointings_list", "pointings_"),
             "-i", "0"]
    return args


def output_names(spec: ProblemSpec, out_prefix: str) -> Dict[str, str]:
    """Output file names the reference writes (sanepic.cc:1618-1690, 1786-1801)."""
    e = f"output_N{spec.nside}_.bin"
    O = out_prefix
    return {
        "I": f"{O}_I_{e}_1", "Q": f"{O}_Q_{e}_1", "U": f"{O}_U_{e}_1",
        "A": f"{O}_A_{e}_1", "NVAR": f"{O}_NVAR{e}", "Q_NVAR": f"{O}_Q_NVAR{e}",
        "U_NVAR": f"{O}_U_NVAR{e}", "HITS": f"{O}_HITS{e}",
        "POL_HITS": f"{O}_POL_HITS{e}", "COS2P": f"{O}_COS2P_{e}",
        "SIN2P": f"{O}_SIN2P_{e}",
    }
