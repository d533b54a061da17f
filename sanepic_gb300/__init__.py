"""sanepic_gb300 -- GB300-native GLS map-maker (the PCG hot path of SANEPIC).

Python mirror of the C ABI in include/sanepic_gpu.h, over ctypes.  The compute
runs only in libsanepic_gpu.so (hand-written sm_103a kernels); if that library
is missing this package raises instead of falling back to anything else.

    mm = MapMaker(ns, nseg, ndet, nside, precision="f32")
    mm.set_pointing(ra, dec, psi, dets)     # boresight timelines + detectors
    mm.set_noise(det, ispf); mm.set_tod(det, tod)
    mm.rhs(); rep = mm.solve(precond="bj3", stop_crit=1e-12)
    I = mm.get_map("I")
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsanepic_gpu.so")

D2PI = 6.2831853071795864769252867665590057683943387987502

SG_OK = 0
SG_ERR_ARG = -1
SG_ERR_UNSUPPORTED = -5
ERRORS = {-1: "SG_ERR_ARG", -2: "SG_ERR_CUDA", -3: "SG_ERR_STATE", -4: "SG_ERR_POINTING",
          -5: "SG_ERR_UNSUPPORTED", -6: "SG_ERR_PRECOND", -7: "SG_ERR_NOT_CONVERGED"}
PRECISION = {"f64": 0, "f32": 1}
PRECOND = {"bj3": 0, "diag": 1, "learned": 2}
MAPS = {"I": 0, "Q": 1, "U": 2, "NVAR": 3, "Q_NVAR": 4, "U_NVAR": 5, "HITS": 6,
        "POL_HITS": 7, "COS2P": 8, "SIN2P": 9}

# every symbol include/sanepic_gpu.h declares
EXPORTS = ["sg_create", "sg_set_stream", "sg_set_pointing", "sg_set_noise", "sg_set_tod", "sg_rhs", "sg_npix",
           "sg_group_mode", "sg_weighting", "sg_kernel_launches",
           "sg_apply", "sg_noise_filter", "sg_noise_filter_noalloc", "sg_solve", "sg_get_map", "sg_get_solution",
           "sg_get_pixels", "sg_get_indpix", "sg_get_crit_history", "sg_profile_operator",
           "sg_learn_train", "sg_learn_nparams", "sg_learn_get_params", "sg_learn_set_params",
           "sg_coarse_from_gram", "sg_mlp_gemm_host", "sg_mlp_grad_host", "sg_solve_batch",
           "sg_autotune", "sg_set_pol_rcond", "sg_tile_shapes", "sg_set_gains", "sg_fit_gains", "sg_set_noise_all", "sg_set_tod_all", "sg_gains_from_sums",
           "sg_last_error", "sg_destroy"]


class SanepicError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SgDesc(ctypes.Structure):
    _fields_ = [("ns", ctypes.c_long), ("nseg", ctypes.c_long), ("ndet", ctypes.c_long),
                ("nside", ctypes.c_long), ("pol", ctypes.c_int), ("hwp", ctypes.c_int),
                ("omega", ctypes.c_double), ("precision", ctypes.c_int),
                ("device", ctypes.c_int)]


class SgDet(ctypes.Structure):
    _fields_ = [("offx", ctypes.c_double), ("offy", ctypes.c_double), ("psi", ctypes.c_double)]


ITER_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                           ctypes.c_double, ctypes.c_double)


class SgSolveOpts(ctypes.Structure):
    _fields_ = [("precond", ctypes.c_int), ("stop_crit", ctypes.c_double),
                ("maxiter", ctypes.c_int), ("refresh_every", ctypes.c_int),
                ("verbose", ctypes.c_int), ("x0", ctypes.POINTER(ctypes.c_double)),
                ("use_graph", ctypes.c_int), ("on_iteration", ITER_CB),
                ("user", ctypes.c_void_p)]


class SgReport(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int),
                ("crit", ctypes.c_double), ("var00", ctypes.c_double),
                ("solve_seconds", ctypes.c_double), ("iter_per_sec", ctypes.c_double),
                ("setup_seconds", ctypes.c_double), ("device_seconds", ctypes.c_double),
                ("kernel_launches", ctypes.c_long), ("breakdown", ctypes.c_int),
                ("fallback_iter", ctypes.c_int), ("crit0", ctypes.c_double)]


class SgLearnOpts(ctypes.Structure):
    _fields_ = [("npairs", ctypes.c_int), ("seed", ctypes.c_long), ("steps", ctypes.c_int),
                ("batch", ctypes.c_int), ("lr", ctypes.c_float), ("pair_crit", ctypes.c_double),
                ("val_crit", ctypes.c_double), ("force", ctypes.c_int),
                ("coarse_k", ctypes.c_int), ("coarse_vectors", ctypes.c_int)]


class SgLearnReport(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_int), ("skies", ctypes.c_int), ("rows", ctypes.c_long),
                ("steps", ctypes.c_int), ("loss_first", ctypes.c_float),
                ("loss_last", ctypes.c_float), ("gen_seconds", ctypes.c_double),
                ("train_seconds", ctypes.c_double), ("gemm_tflop", ctypes.c_double),
                ("val_plain_iters", ctypes.c_int), ("val_learned_iters", ctypes.c_int),
                ("val_plain_ms", ctypes.c_double), ("val_learned_ms", ctypes.c_double),
                ("enabled", ctypes.c_int), ("coarse_k", ctypes.c_int),
                ("coarse_vectors", ctypes.c_int), ("coarse_seconds", ctypes.c_double),
                ("val_coarse_iters", ctypes.c_int), ("val_coarse_ms", ctypes.c_double),
                ("kind", ctypes.c_int)]


_lib = None


def load_library(path: Optional[str] = None):
    """Load libsanepic_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with sanepic_gb300.build.build() "
                           "(there is no CPU fallback)")
    L = ctypes.CDLL(p)
    c_p = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    lp = ctypes.POINTER(ctypes.c_long)
    L.sg_create.argtypes = [ctypes.POINTER(c_p), ctypes.POINTER(SgDesc)]
    L.sg_set_stream.argtypes = [c_p, c_p]
    L.sg_set_pointing.argtypes = [c_p, dp, dp, dp, ctypes.c_long, lp, ctypes.POINTER(SgDet)]
    L.sg_set_noise.argtypes = [c_p, ctypes.c_long, dp, ctypes.c_long]
    L.sg_set_noise_all.argtypes = [c_p, dp, ctypes.c_long]
    L.sg_set_tod_all.argtypes = [c_p, dp, ctypes.c_long]
    L.sg_set_pol_rcond.argtypes = [c_p, ctypes.c_double]
    L.sg_tile_shapes.argtypes = [c_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.sg_set_tod.argtypes = [c_p, ctypes.c_long, dp, ctypes.c_long]
    L.sg_rhs.argtypes = [c_p, dp]
    L.sg_set_gains.argtypes = [c_p, dp]
    L.sg_fit_gains.argtypes = [c_p, ctypes.c_int, dp, dp, dp]
    L.sg_gains_from_sums.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_int, dp, dp, dp, dp,
                                     dp, dp, dp]
    L.sg_npix.argtypes = [c_p]
    L.sg_npix.restype = ctypes.c_long
    L.sg_group_mode.argtypes = [c_p, ctypes.POINTER(ctypes.c_long)]
    L.sg_group_mode.restype = ctypes.c_int
    L.sg_weighting.argtypes = [c_p]
    L.sg_weighting.restype = ctypes.c_int
    L.sg_kernel_launches.argtypes = [c_p]
    L.sg_kernel_launches.restype = ctypes.c_long
    L.sg_apply.argtypes = [c_p, dp, dp, ctypes.c_int]
    L.sg_noise_filter.argtypes = [c_p, dp, dp]
    L.sg_noise_filter_noalloc.argtypes = [c_p, c_p, c_p, ctypes.c_long, ctypes.c_long,
                                          ctypes.c_long, c_p]
    L.sg_solve.argtypes = [c_p, ctypes.POINTER(SgSolveOpts), ctypes.POINTER(SgReport)]
    L.sg_get_map.argtypes = [c_p, ctypes.c_int, dp]
    L.sg_get_solution.argtypes = [c_p, dp]
    L.sg_get_pixels.argtypes = [c_p, lp]
    L.sg_get_indpix.argtypes = [c_p, lp]
    L.sg_get_crit_history.argtypes = [c_p, dp, ctypes.c_int]
    L.sg_profile_operator.argtypes = [c_p, ctypes.c_int, dp]
    fp = ctypes.POINTER(ctypes.c_float)
    L.sg_learn_train.argtypes = [c_p, ctypes.POINTER(SgLearnOpts), ctypes.POINTER(SgLearnReport)]
    L.sg_learn_nparams.argtypes = []
    L.sg_learn_nparams.restype = ctypes.c_long
    L.sg_learn_get_params.argtypes = [c_p, fp]
    L.sg_learn_set_params.argtypes = [c_p, fp]
    dp = ctypes.POINTER(ctypes.c_double)
    L.sg_coarse_from_gram.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp]
    L.sg_coarse_from_gram.restype = ctypes.c_int
    L.sg_mlp_gemm_host.argtypes = [ctypes.POINTER(ctypes.c_ushort), ctypes.POINTER(ctypes.c_ushort),
                                   fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    L.sg_mlp_grad_host.argtypes = [fp, fp, fp, ctypes.c_int, fp, fp, fp]
    L.sg_solve_batch.argtypes = [ctypes.POINTER(c_p), ctypes.c_int, ctypes.POINTER(SgSolveOpts),
                                 ctypes.POINTER(SgReport)]
    L.sg_autotune.argtypes = [c_p, ctypes.POINTER(ctypes.c_int), dp]
    L.sg_last_error.argtypes = [c_p]
    L.sg_last_error.restype = ctypes.c_char_p
    L.sg_destroy.argtypes = [c_p]
    if path is None:
        _lib = L
    return L


def _fp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class MapMaker:
    """One map-making problem on one GPU (a context of the C ABI)."""

    def __init__(self, ns: int, nseg: int, ndet: int, nside: int, hwp: bool = False,
                 omega: float = 0.0, precision: str = "f32", device: int = 0):
        self.L = load_library()
        self.ns, self.nseg, self.ndet, self.nside = ns, nseg, ndet, nside
        self.precision = precision
        self.device = device
        desc = SgDesc(ns, nseg, ndet, nside, 1, int(bool(hwp)), float(omega),
                      PRECISION[precision], device)
        h = ctypes.c_void_p()
        rc = self.L.sg_create(ctypes.byref(h), ctypes.byref(desc))
        self.h = h
        if rc != SG_OK:
            msg = self.L.sg_last_error(h).decode() if h.value else "sg_create failed"
            self.close()
            raise SanepicError(rc, msg)

    def _check(self, rc: int):
        if rc < 0:
            raise SanepicError(rc, self.L.sg_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.sg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: Optional[int]):
        """Run on an existing cudaStream_t (an integer handle), None = own stream."""
        self._check(self.L.sg_set_stream(self.h, ctypes.c_void_p(stream_handle or None)))

    # ---- inputs -----------------------------------------------------------
    def set_pointing(self, ra, dec, psi, dets: Sequence, isampmin=None):
        ra, dec, psi = _f64(ra), _f64(dec), _f64(psi)
        arr = (SgDet * self.ndet)(*[SgDet(*map(float, d)) for d in dets])
        isp = None
        if isampmin is not None:
            self._isamp = np.ascontiguousarray(isampmin, dtype=np.int64)
            isp = self._isamp.ctypes.data_as(ctypes.POINTER(ctypes.c_long))
        self._check(self.L.sg_set_pointing(self.h, _dp(ra), _dp(dec), _dp(psi), ra.size, isp, arr))
        self.npix = int(self.L.sg_npix(self.h))

    def set_pol_rcond(self, rcond_min: float):
        """Also mask Q/U where the pixel's 3 x 3 hit block has a reciprocal
        condition number below rcond_min (0: the reference's rule only)."""
        self._check(self.L.sg_set_pol_rcond(self.h, float(rcond_min)))

    def set_noise(self, det: int, ispf):
        ispf = _f64(ispf)
        self._check(self.L.sg_set_noise(self.h, det, _dp(ispf), ispf.size))

    def set_noise_all(self, ispf):
        """Every detector's iSpf at once: ispf [ndet][nssp]."""
        ispf = _f64(ispf)
        if ispf.ndim != 2 or ispf.shape[0] != self.ndet:
            raise ValueError(f"ispf: want [{self.ndet}][nssp], got {ispf.shape}")
        self._check(self.L.sg_set_noise_all(self.h, _dp(ispf), ispf.shape[1]))

    def set_tod(self, det: int, tod):
        tod = _f64(tod)
        self._check(self.L.sg_set_tod(self.h, det, _dp(tod), tod.size))

    def set_tod_all(self, tod):
        """Every detector's timeline at once: tod [ndet][nsamp_total]."""
        tod = _f64(tod)
        if tod.ndim != 2 or tod.shape[0] != self.ndet:
            raise ValueError(f"tod: want [{self.ndet}][nsamp], got {tod.shape}")
        self._check(self.L.sg_set_tod_all(self.h, _dp(tod), tod.shape[1]))

    # ---- recalibration (sanepic.cc:1041-1130, 2123-2316) ---------------------
    def set_gains(self, gains) -> None:
        """Per-tile gains [nseg][ndet] (the reference's relCalib layout), or
        None for 1; the next rhs() and solve() use them."""
        if gains is None:
            self._check(self.L.sg_set_gains(self.h, None))
            return
        g = _f64(gains)
        if g.size != self.nseg * self.ndet:
            raise ValueError(f"gains: {g.size} values for {self.nseg} x {self.ndet} tiles")
        self._check(self.L.sg_set_gains(self.h, _dp(g)))

    def fit_gains(self, per_detector: bool = False):
        """Gains refitted to the current map: (gains [nseg][ndet], chi2 before,
        chi2 after).  Not applied; pass them to set_gains()."""
        g = np.empty(self.nseg * self.ndet)
        b = ctypes.c_double(0.0)
        a = ctypes.c_double(0.0)
        self._check(self.L.sg_fit_gains(self.h, int(per_detector), _dp(g), ctypes.byref(b),
                                        ctypes.byref(a)))
        return g.reshape(self.nseg, self.ndet), b.value, a.value

    def recalibrate(self, precond: str = "bj3", stop_crit: float = 1e-15, maxiter: int = 2000,
                    per_detector: bool = False, max_loops: int = 499) -> dict:
        """The reference's -r (-R: per_detector) outer loop (sanepic.cc:1041-1042,
        2123-2316), as the drop-in executable runs it: make the map with gains
        1, fit the gains to it, make the map again from the previous one with
        the new gains, until a loop starts already converged (its var0 / var00
        at most stop_crit, var00 of the first loop) or after max_loops loops.
        Returns the last fitted gains [nseg][ndet], the loops made, chi^2
        (before, after) of every fit and the iterations of every solve; the
        map is the last loop's."""
        self.set_gains(None)
        self.rhs(chi2=False)
        rep = self.solve(precond=precond, stop_crit=stop_crit, maxiter=maxiter)
        var00 = rep["var00"]
        ratio = rep["crit0"]
        chi2, iters = [], [rep["iterations"]]
        loops = 1
        while True:
            g, before, after = self.fit_gains(per_detector)
            chi2.append((before, after))
            if not (loops < max_loops and ratio > stop_crit):
                break
            loops += 1
            self.set_gains(g)
            self.rhs(chi2=False)
            rep = self.solve(precond=precond, stop_crit=stop_crit, maxiter=maxiter,
                             x0=self.solution())
            ratio = rep["crit0"] * rep["var00"] / var00
            iters.append(rep["iterations"])
        return {"gains": g, "loops": loops, "chi2": chi2, "iterations": iters}

    # ---- operator -----------------------------------------------------------
    def rhs(self, chi2: bool = True) -> Optional[float]:
        """b = P^T N^-1 d; returns chi2_0, or None with chi2=False (then groups
        of detectors with one noise spectrum skip the per-detector FFTs)."""
        if not chi2:
            self._check(self.L.sg_rhs(self.h, None))
            return None
        c = ctypes.c_double(0.0)
        self._check(self.L.sg_rhs(self.h, ctypes.byref(c)))
        return c.value

    def apply(self, x, masked: bool = False) -> np.ndarray:
        x = _f64(x)
        y = np.empty(3 * self.npix)
        self._check(self.L.sg_apply(self.h, _dp(x), _dp(y), int(masked)))
        return y

    def noise_filter(self, arr) -> np.ndarray:
        a = _f64(arr).reshape(-1)
        out = np.empty_like(a)
        self._check(self.L.sg_noise_filter(self.h, _dp(a), _dp(out)))
        return out

    def solve(self, precond: str = "bj3", stop_crit: float = 1e-15, maxiter: int = 2000,
              refresh_every: int = 10, verbose: bool = False, x0=None,
              use_graph: bool = True, on_iteration=None, history: bool = False) -> dict:
        """Run PCG.  on_iteration(iter, crit, crit2, chi2) -> bool (True
        stops) runs after each iteration; with history=True the report also
        holds `history`, one (iter, crit, crit2, chi2) row per iteration (the
        reference's printed line).  chi^2 of the refresh iterations is computed
        only when a callback, history or verbose asks for it."""
        x0p = None
        if x0 is not None:
            self._x0 = _f64(x0)
            x0p = _dp(self._x0)
        hist = []

        def _cb(_user, it, crit, crit2, chi2):
            hist.append((it, crit, crit2, chi2))
            return int(bool(on_iteration(it, crit, crit2, chi2))) if on_iteration else 0

        cb = ITER_CB(_cb) if (on_iteration or history) else ITER_CB()
        o = SgSolveOpts(PRECOND[precond], stop_crit, maxiter, refresh_every, int(verbose),
                        x0p, int(use_graph), cb, None)
        rep = SgReport()
        self._check(self.L.sg_solve(self.h, ctypes.byref(o), ctypes.byref(rep)))
        out = {k: getattr(rep, k) for k, _ in SgReport._fields_}
        if history:
            out["history"] = np.array(hist, dtype=np.float64).reshape(-1, 4)
        return out

    # ---- outputs ------------------------------------------------------------
    def get_map(self, kind: str) -> np.ndarray:
        out = np.empty(12 * self.nside * self.nside)
        self._check(self.L.sg_get_map(self.h, MAPS[kind], _dp(out)))
        return out

    def solution(self) -> np.ndarray:
        out = np.empty(3 * self.npix)
        self._check(self.L.sg_get_solution(self.h, _dp(out)))
        return out

    def pixels(self) -> np.ndarray:
        out = np.empty(self.ndet * self.nseg * self.ns, dtype=np.int64)
        self._check(self.L.sg_get_pixels(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_long))))
        return out

    def indpix(self) -> np.ndarray:
        out = np.empty(12 * self.nside * self.nside, dtype=np.int64)
        self._check(self.L.sg_get_indpix(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_long))))
        return out

    def group_mode(self):
        """(True if the operator runs per offset group, number of groups)"""
        n = ctypes.c_long(0)
        on = bool(self.L.sg_group_mode(self.h, ctypes.byref(n)))
        return on, int(n.value)

    def kernel_launches(self) -> int:
        """Kernels this context has launched so far (graph nodes one by one)."""
        return int(self.L.sg_kernel_launches(self.h))

    def weighting(self) -> str:
        """How the operator applies N^-1: "per-detector" (one fused cluster
        filter per detector timeline), "group" (cluster FFT kernels on the
        offset groups' three timelines), with "-3pass" where the three-pass
        FP32 FFT through L2 runs instead.  Known once the operator was
        prepared."""
        w = self.L.sg_weighting(self.h)
        return ("group" if w & 1 else "per-detector") + ("-3pass" if w & 2 else "")

    def autotune(self) -> dict:
        """Pick the faster compiled FFT tile shape for this problem's noise filter."""
        S = ctypes.c_int(0)
        ms = ctypes.c_double(0.0)
        self._check(self.L.sg_autotune(self.h, ctypes.byref(S), ctypes.byref(ms)))
        lanes = ctypes.c_int(0)
        self._check(self.L.sg_tile_shapes(self.h, ctypes.byref(S), ctypes.byref(lanes)))
        return {"cluster_size": S.value, "filter_ms": ms.value, "pt_lanes": lanes.value}

    # ---- learned preconditioner ---------------------------------------------
    def learn_train(self, npairs: int = 512, seed: int = 5000, steps: int = 1500,
                    batch: int = 0, lr: float = 1e-3, pair_crit: float = 1e-13,
                    val_crit: float = 1e-12, force=False, coarse_k: int = 0,
                    coarse_vectors: int = 0) -> dict:
        """Make residual/solution pairs with the plain solver on synthetic skies,
        build the coarse space and train the network on the GPU, and validate
        both against plain PCG on a held-out problem (steps < 0: no network;
        coarse_k < 0: no coarse space).  force: True or "network" uses the
        network, "coarse" the coarse space, even without a validated gain.
        Overwrites b: call rhs() again."""
        fcode = {False: 0, None: 0, True: 1, "network": 1, "coarse": 2}[force]
        o = SgLearnOpts(npairs, seed, steps, batch, lr, pair_crit, val_crit, fcode,
                        coarse_k, coarse_vectors)
        rep = SgLearnReport()
        self._check(self.L.sg_learn_train(self.h, ctypes.byref(o), ctypes.byref(rep)))
        return {k: getattr(rep, k) for k, _ in SgLearnReport._fields_}

    def learn_params(self) -> np.ndarray:
        out = np.empty(int(self.L.sg_learn_nparams()), dtype=np.float32)
        self._check(self.L.sg_learn_get_params(self.h, _fp(out)))
        return out

    def set_learn_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.L.sg_learn_set_params(self.h, _fp(p)))

    def profile_operator(self, reps: int = 5) -> dict:
        ms = np.zeros(4)
        self._check(self.L.sg_profile_operator(self.h, reps, _dp(ms)))
        return {"p_ms": float(ms[0]), "filter_ms": float(ms[1]), "detsum_ms": float(ms[2]),
                "pt_ms": float(ms[3])}

    def crit_history(self, max_n: int = 100000) -> np.ndarray:
        out = np.empty(max_n)
        n = self._check(self.L.sg_get_crit_history(self.h, _dp(out), max_n))
        return out[:n].copy()


def noise_filter_noalloc(in_ptr: int, out_ptr: int, filt_ptr: int, ns: int, ntiles: int,
                         tiles_per_filter: int, stream: Optional[int] = None) -> int:
    """sg_noise_filter_noalloc on raw device pointers (FP32): N^-1 applied to
    caller-owned device buffers without any GPU allocation.  Returns the C
    status code (0 on success)."""
    L = load_library()
    return L.sg_noise_filter_noalloc(ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr),
                                     ctypes.c_void_p(filt_ptr), ns, ntiles, tiles_per_filter,
                                     ctypes.c_void_p(stream or None))


def detectors_from_angles(angles_deg, offsets=None):
    """sg_det rows (offx, offy, psi) as the reference derives them
    (sanepic.cc:458-463): zero offsets unless given, psi = angle in radians."""
    rows = []
    for d, a in enumerate(angles_deg):
        ox, oy = (0.0, 0.0) if offsets is None else offsets[d]
        rows.append((ox, oy, float(a) / 180.0 * D2PI / 2.0))
    return rows


def from_problem(prob, precision: Optional[str] = None, device: int = 0,
                 with_tod: bool = True) -> MapMaker:
    """A MapMaker loaded with an in-memory problem (see sanepic_gb300.synth)."""
    spec = prob["spec"]
    prec = precision or spec.precision
    mm = MapMaker(spec.ns, spec.nseg, spec.ndet, spec.nside, hwp=spec.hwp,
                  omega=prob["omega"], precision=prec, device=device)
    mm.set_pointing(prob["ra"], prob["dec"], prob["psi"], detectors_from_angles(prob["angles"]),
                    prob.get("isampmin"))
    for d in range(spec.ndet):
        mm.set_noise(d, prob["ispf"][d])
        if with_tod and "tod" in prob:
            mm.set_tod(d, prob["tod"][d])
    return mm


def gains_from_sums(dots_ds, dots_ss, edges_s, edges_d, spn_edge, g_old, per_detector=False):
    """sg_fit_gains' host arithmetic on given per-tile sums (no GPU): arrays
    [ndet][nseg] (edges [ndet][nseg][2], spn_edge [ndet][2]); returns the new
    gains [ndet][nseg]."""
    g_old = _f64(g_old)
    ndet, nseg = g_old.shape
    out = np.empty_like(g_old)
    args = [_f64(a) for a in (dots_ds, dots_ss, edges_s, edges_d, spn_edge)]
    rc = load_library().sg_gains_from_sums(ndet, nseg, int(per_detector), *[_dp(a) for a in args],
                                           _dp(g_old), _dp(out))
    if rc != SG_OK:
        raise SanepicError(rc, "no positive mean gain")
    return out


# ---- tensor-core GEMM and network gradients on host arrays (tests, measurements) ----
def coarse_from_gram(H: np.ndarray, G: np.ndarray, kc: int):
    """The coarse space's Rayleigh-Ritz step on host arrays (no GPU): returns
    (C [m][k], E^-1 [k][k], theta [k]) for H = V^T A V, G = V^T M^-1 V."""
    H = np.ascontiguousarray(H, np.float64)
    G = np.ascontiguousarray(G, np.float64)
    m = H.shape[0]
    C = np.zeros((m, kc))
    einv = np.zeros((kc, kc))
    th = np.zeros(kc)
    k = int(load_library().sg_coarse_from_gram(m, kc, _dp(H), _dp(G), _dp(C), _dp(einv),
                                               _dp(th)))
    return (C.reshape(-1)[:m * k].reshape(m, k), einv.reshape(-1)[:k * k].reshape(k, k),
            th[:k])


def mlp_nparams() -> int:
    return int(load_library().sg_learn_nparams())


def gemm_bf16(a_bits: np.ndarray, b_bits: np.ndarray, reps: int = 0):
    """C = A . B^T for BF16 bit patterns A [M, K], B [N, K] (uint16).  Returns
    (C float32 [M, N], mean milliseconds per GEMM when reps > 0)."""
    A = np.ascontiguousarray(a_bits, dtype=np.uint16)
    B = np.ascontiguousarray(b_bits, dtype=np.uint16)
    M, K = A.shape
    N = B.shape[0]
    C = np.empty((M, N), dtype=np.float32)
    ms = ctypes.c_double(0.0)
    rc = load_library().sg_mlp_gemm_host(A.ctypes.data_as(ctypes.POINTER(ctypes.c_ushort)),
                                         B.ctypes.data_as(ctypes.POINTER(ctypes.c_ushort)),
                                         _fp(C), M, N, K, reps, ctypes.byref(ms))
    if rc:
        raise SanepicError(rc, "sg_mlp_gemm_host failed")
    return C, ms.value


def mlp_grad(params: np.ndarray, X: np.ndarray, T: np.ndarray):
    """One forward + backward of the network: returns (Y, loss, grads)."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    Y = np.empty_like(X)
    g = np.empty_like(p)
    loss = ctypes.c_float(0.0)
    rc = load_library().sg_mlp_grad_host(_fp(p), _fp(X), _fp(T), X.shape[0], _fp(Y),
                                         ctypes.byref(loss), _fp(g))
    if rc:
        raise SanepicError(rc, "sg_mlp_grad_host failed")
    return Y, float(loss.value), g


def solve_batch(makers, precond: str = "bj3", stop_crit: float = 1e-15, maxiter: int = 2000,
                refresh_every: int = 10, use_graph: bool = True) -> list:
    """Solve several MapMakers (each after rhs()) concurrently, one CUDA stream
    each; returns one report dict per problem (as MapMaker.solve)."""
    L = load_library()
    n = len(makers)
    hs = (ctypes.c_void_p * n)(*[m.h.value for m in makers])
    o = SgSolveOpts(PRECOND[precond], stop_crit, maxiter, refresh_every, 0, None,
                    int(use_graph), ITER_CB(), None)
    reps = (SgReport * n)()
    rc = L.sg_solve_batch(hs, n, ctypes.byref(o), reps)
    if rc:
        raise SanepicError(rc, L.sg_last_error(makers[0].h).decode())
    return [{k: getattr(r, k) for k, _ in SgReport._fields_} for r in reps]
