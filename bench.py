#!/usr/bin/env python3
"""Benchmark: time-to-solution of the GLS map-making PCG on one GB300,
learned-preconditioned (flexible PCG) against plain block-Jacobi PCG.

The learned mode applies whichever learned part plain PCG judged faster on a
held-out problem: the coarse space (Ritz vectors of M A from the plain
solver's own residuals, two-level balancing preconditioner) or the patch
network; if neither gained it runs plain block-Jacobi PCG and says so.

Workload (default): 64 detectors, NSIDE 256, 48 segments x 131,072 samples
(4.03e8 samples), FP32 operator with FP64 P^T sums and CG scalars, seeded
synthetic scan/sky/1-over-f noise (sanepic_gb300.synth).  One step = one
solve from x0 = 0 to |r|/|b| <= 1e-6 (crit = |r|^2/|b|^2 <= 1e-12):
  value: b = P^T N^-1 d (sg_rhs without chi2_0, a diagnostic; detectors
         sharing pointing and noise spectrum are then summed before the
         FFTs) plus the PCG in the learned-preconditioner mode,
         inputs already resident in HBM, CUDA-event time on the library's
         stream (the bench's torch stream).  The network is trained and
         judged by plain PCG before the timed region (training time is
         reported, not timed); if it lost on its held-out validation problem
         the learned mode runs plain block-Jacobi PCG and the line says so;
  plain: the same steps with plain block-Jacobi PCG;
  e2e:   a solve through the C ABI from host buffers: pointing, noise and
         TOD uploaded (host->device) every step, maps read back.
The operator kernels (P, the noise filter, the per-group detector sums, P^T)
are timed live with CUDA events for the roofline against their algorithmic
bytes; the network's tensor-core GEMM is timed against the measured BF16 peak.

--impl reference times the reference's path on the host cores for the whole
workload: the threaded port of sanepic.cc's algorithm (oracle/cgpar.c: the
FP64 restatement in the reference's parallel layout, its diagonal
preconditioner and PCG), each run from scratch to |r|/|b| <= 1e-6.  The
reference binary itself is built only where its source is (not on the GPU
host); oracle/calibrate_port.py times it against the port on one host.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from sanepic_gb300 import synth  # noqa: E402

METRIC = "time-to-solution at rel. residual 1e-6: learned-precond vs plain PCG, 1 GB300"
STOP_CRIT = 1e-12  # |r|^2/|b|^2, i.e. |r|/|b| = 1e-6
# DRAM bytes (read + write) of one noise-filter tile of 131072 FP32 samples,
# from the ncu capture in profiles/noise_filter_c2_8det.md (354.5 MB over
# 384 tiles); traffic grows with the tiles, so a full launch is this x tiles.
FILTER_DRAM_BYTES_PER_TILE_131072_F32 = 354.46e6 / 384
# DRAM bytes (read + write) of one group noise weighting (the three in-place
# passes: columns, rows with the 3 x 3 mixing, inverse columns) on the bench
# workloads with one group of 48 x 131072 samples, L2 as the operator's
# previous kernel left it, from the ncu capture in
# profiles/group_noise_weighting_c2_8det.md (273.2 MB with the caches flushed
# before each launch)
GROUP_NW_DRAM_BYTES = {("c2_64det_nside256", "f32"): 208.1e6, ("c2_8det_nside256", "f32"): 208.1e6}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (every 200 ms) during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        if shutil.which("nvidia-smi") is None:
            return self
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        self.proc = subprocess.Popen(
            ["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
             "--format=csv,noheader,nounits", "-lms", "200"],
            stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                "sw_power_cap"), f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(sec, device):
    """The slowest rank's time: every rank runs its own replica of the
    workload (the path has no exchange step), and the job takes as long as
    its slowest replica.  One process: sec itself."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return sec
    t = torch.tensor([sec], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    import sanepic_gb300 as sg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    spec = synth.spec_from_name(args.config)
    t0 = time.time()
    prob = synth.make_problem(spec)
    gen_s = time.time() - t0
    stream = torch.cuda.current_stream()
    dets = sg.detectors_from_angles(prob["angles"])

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def upload(mm):
        mm.set_pointing(prob["ra"], prob["dec"], prob["psi"], dets, prob["isampmin"])
        for d in range(spec.ndet):
            mm.set_noise(d, prob["ispf"][d])
            mm.set_tod(d, prob["tod"][d])

    mm = sg.MapMaker(spec.ns, spec.nseg, spec.ndet, spec.nside, hwp=spec.hwp,
                     omega=prob["omega"], precision=spec.precision, device=local)
    mm.set_stream(stream.cuda_stream)
    upload(mm)

    def device_step(precond):
        mm.rhs(chi2=False)  # b only: chi2_0 is a diagnostic, not part of the solution
        return mm.solve(precond=precond, stop_crit=STOP_CRIT, maxiter=args.maxiter)

    # ---- the learned preconditioner: trained and judged before timing --------
    learn = None
    precond = args.precond
    if not args.no_learn:
        tl = time.time()
        learn = mm.learn_train(npairs=args.learn_pairs, steps=args.learn_steps,
                               coarse_k=args.coarse_k, coarse_vectors=args.coarse_vectors)
        learn["wall_seconds"] = time.time() - tl
        precond = "learned"

    def timed(pc, clk=None):
        for _ in range(args.warmup):
            device_step(pc)
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = []
        # an NVTX range marks the timed steps for profilers (ncu --nvtx)
        torch.cuda.nvtx.range_push(f"timed_{pc}")
        # the library's own count of the kernels it launches (RHS and solve;
        # graph nodes one by one)
        launches0 = mm.kernel_launches()
        ev0.record(stream)
        for _ in range(args.steps):
            rep = device_step(pc)
            reps.append(rep)
        ev1.record(stream)
        launches = mm.kernel_launches() - launches0
        torch.cuda.nvtx.range_pop()
        barrier()
        sec = max_over_ranks(ev0.elapsed_time(ev1) / args.steps / 1e3, "cuda")
        return sec, reps, launches

    # ---- value: inputs resident, CUDA events on the launching stream -------
    with ClockSampler(local) as clk:
        sec, reps, launches = timed(precond)
        if learn is not None:
            sec_plain, reps_plain, _ = timed(args.precond)
    clocks = clk.summary()
    iters = reps[-1]["iterations"]
    # ---- roofline of the dominant kernel (same stream, live) -----------------
    prof = mm.profile_operator(reps=5)
    ns_all = spec.ndet * spec.nseg * spec.ns
    npix = mm.npix
    esz = 4 if spec.precision == "f32" else 8
    # algorithmic bytes per launch (each input read once, each output written once).
    # Detectors sharing focal-plane offsets share one pixel stream: pixel index,
    # base angle and the CSR live per group sample (ng), y per detector sample.
    group, ngrp = mm.group_mode()  # the synthetic detectors all sit on the boresight
    ng = ngrp * spec.nseg * spec.ns
    m1 = spec.ns // 2 + 1
    pt_bytes = ng * (4 + 2 * esz + 4 * esz) + npix * (3 * 8 + 8 + 4)
    if group:
        # per offset group: (a, b1, b2) per group sample; N^-1 = the three
        # in-place passes (column FFTs, row FFTs with the 3 x 3 mixing,
        # inverse column FFTs; three launches, timed together): the three
        # timelines read, the three weighted ones written, the mixing
        # matrices read; the passes' round trips through L2 are not
        # algorithmic
        kbytes = {
            "k_group_project": ng * (4 + 2 * esz) + npix * 4 * esz + 3 * ng * esz,
            "group_noise_weighting": 6 * ng * esz + ngrp * m1 * 6 * esz,
            "k_pt": pt_bytes,
        }
        kms = {"k_group_project": prof["p_ms"], "group_noise_weighting": prof["filter_ms"],
               "k_pt": prof["pt_ms"]}
    else:
        kbytes = {
            "k_project": ng * (4 + 2 * esz) + ns_all * esz + npix * 4 * esz,
            "k_noise_filter": ns_all * 2 * esz + spec.ndet * m1 * esz,
            "k_detsum": ns_all * esz + ng * 4 * esz,
            "k_pt": pt_bytes,
        }
        kms = {"k_project": prof["p_ms"], "k_noise_filter": prof["filter_ms"],
               "k_detsum": prof["detsum_ms"], "k_pt": prof["pt_ms"]}
    hbm, peak_kind = peaks()
    kernels = {k: {"ms": kms[k], "GBps": kbytes[k] / (kms[k] * 1e-3) / 1e9,
                   "bytes": kbytes[k]} for k in kbytes}
    dom = max(kms, key=kms.get)
    achieved = kernels[dom]["GBps"]
    traffic = None
    if dom == "k_noise_filter" and spec.ns == 131072 and spec.precision == "f32":
        traffic = FILTER_DRAM_BYTES_PER_TILE_131072_F32 * spec.ndet * spec.nseg
    if (dom == "group_noise_weighting" and mm.weighting() == "group-3pass"
            and (args.config, spec.precision) in GROUP_NW_DRAM_BYTES):
        traffic = GROUP_NW_DRAM_BYTES[(args.config, spec.precision)]
    # ---- accuracy of the timed solves: maps against an FP64 solve -----------
    extra = {}
    if not args.no_map_error:
        extra["map_error"] = map_error(sg, mm, spec, prob, dets, precond, stream, args)
    # ---- plain block-Jacobi vs the reference's diagonal (same workload) -------
    if args.compare_diag:
        rep_d = device_step("diag")
        extra["diag_precond"] = {"iterations": rep_d["iterations"],
                                 "seconds": rep_d["device_seconds"],
                                 "converged": bool(rep_d["converged"])}
        device_step(args.precond)
    # ---- e2e through the C ABI with host buffers ------------------------------
    # the step's inputs sit in pinned (page-locked) host memory, as a caller
    # streaming observations would hold them
    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        out = t.numpy()
        out[...] = a
        return out

    host = {k: pinned(prob[k]) for k in ("ra", "dec", "psi", "ispf", "tod")}
    h2d = (3 * prob["ra"].size * 8 + spec.ndet * prob["ispf"][0].size * 8
           + spec.ndet * prob["tod"][0].size * 8)
    d2h = 3 * 12 * spec.nside ** 2 * 8
    e2e, phases = [], []
    for i in range(args.e2e_steps):
        barrier()
        nvtx = torch.cuda.nvtx
        te = time.perf_counter()
        nvtx.range_push("e2e_pointing")
        mm.set_pointing(host["ra"], host["dec"], host["psi"], dets, prob["isampmin"])
        nvtx.range_pop()
        t1 = time.perf_counter()
        nvtx.range_push("e2e_noise")
        mm.set_noise_all(host["ispf"])  # one copy for every detector's spectrum
        nvtx.range_pop()
        t2 = time.perf_counter()
        nvtx.range_push("e2e_tod")
        mm.set_tod_all(host["tod"])  # every detector's timeline, one wait
        nvtx.range_pop()
        t3 = time.perf_counter()
        nvtx.range_push("e2e_solve")
        device_step(precond)
        nvtx.range_pop()
        t4 = time.perf_counter()
        nvtx.range_push("e2e_maps")
        maps = [mm.get_map(k) for k in ("I", "Q", "U")]
        nvtx.range_pop()
        barrier()
        t5 = time.perf_counter()
        e2e.append(t5 - te)
        phases.append([t1 - te, t2 - t1, t3 - t2, t4 - t3, t5 - t4])
    e2e_s = float(np.median(e2e)) if e2e else None
    e2e_phases = (dict(zip(("pointing", "noise", "tod", "rhs_and_solve", "maps"),
                           np.median(np.array(phases), axis=0).tolist())) if phases else None)
    line = {
        "metric": METRIC, "value": sec, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": spec.precision == "f32" and "f32" or "f64",
        "data": "synthetic (seeded spin+precession scan, iid sky, 1/f noise)",
        "config": {"workload": args.config, "ndet": spec.ndet, "nside": spec.nside,
                   "nseg": spec.nseg, "ns": spec.ns, "samples": ns_all, "npix_obs": npix,
                   "precond": args.precond, "stop": "|r|/|b| <= 1e-6",
                   "iterations": iters, "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "l2": "inputs larger than L2 (pointing alone %.1f GB)" % (ns_all * 12 / 1e9)},
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "phases_s": e2e_phases},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "kernel": dom,
                     "peak_kind": peak_kind, "kernels": kernels},
        "clocks": clocks,
        "iter_per_sec": reps[-1]["iter_per_sec"],
        "generation_s": gen_s,
    }
    line.update(extra)
    if learn is not None:
        line["config"]["precond"] = "learned (flexible PCG, judged by block-Jacobi PCG)"
        kind = {0: "none: plain block-Jacobi PCG", 1: "patch network",
                2: "coarse space"}[learn["kind"]]
        line["learned"] = {
            "plain_pcg_s": sec_plain, "plain_iterations": reps_plain[-1]["iterations"],
            "learned_iterations": iters, "learned_part": kind,
            "network_used": learn["kind"] == 1,
            "fell_back_at_iteration": reps[-1]["fallback_iter"],
            "validation": {"plain_iterations": learn["val_plain_iters"],
                           "network_iterations": learn["val_learned_iters"],
                           "coarse_iterations": learn["val_coarse_iters"],
                           "plain_ms": learn["val_plain_ms"],
                           "network_ms": learn["val_learned_ms"],
                           "coarse_ms": learn["val_coarse_ms"]},
            "coarse_space": {"vectors": learn["coarse_k"],
                             "from_residuals": learn["coarse_vectors"],
                             "build_s": learn["coarse_seconds"],
                             "method": "Rayleigh-Ritz of M_bj3 A on span{M_bj3 r_k}; "
                                       "two-level balancing preconditioner"},
            "training": {"pairs": learn["pairs"], "skies": learn["skies"],
                         "steps": learn["steps"], "loss_first": learn["loss_first"],
                         "loss_last": learn["loss_last"],
                         "pair_generation_s": learn["gen_seconds"],
                         "train_s": learn["train_seconds"],
                         "tensor_core_tflop": learn["gemm_tflop"],
                         "loss": "-(r.z)^2/((z.Az)(r.M r)), A-cosine of the corrected direction"},
        }
        line["mlp_gemm"] = mlp_gemm_roofline(sg, mm)
    if not args.no_per_detector:
        line["per_detector"] = per_detector(sg, spec, prob, dets, stream, args)
    if args.c3 and spec.name != C3:
        mm.close()
        line["c3"] = c3_block(sg, stream, args)
    if not args.no_cpu_baseline and rank == 0:
        line["cpu_baseline"] = reference_cpu(args, spec)
    if rank == 0:
        print(json.dumps(line), flush=True)
    mm.close()
    if world > 1:
        torch.distributed.destroy_process_group()


C3 = "c3_256det_nside512_hwp"


def _map_errs(x, want, npix):
    """Per map: max and RMS error of compact x against want, relative to
    want's max |.| and RMS, also with the mean difference removed (the bin-0
    override of sanepic.cc:536-537 leaves the I monopole nearly free)."""
    out = {}
    for c, k in enumerate("IQU"):
        w = want[c * npix:(c + 1) * npix]
        d = x[c * npix:(c + 1) * npix] - w
        d0 = d - d.mean()
        rw, mw = float(np.sqrt(np.mean(w * w))), float(np.max(np.abs(w)))
        out[k] = {"rms": float(np.sqrt(np.mean(d * d))) / rw, "max": float(np.max(np.abs(d))) / mw,
                  "rms_monopole_removed": float(np.sqrt(np.mean(d0 * d0))) / rw,
                  "max_monopole_removed": float(np.max(np.abs(d0))) / mw}
    return out


def map_error(sg, mm, spec, prob, dets, precond, stream, args):
    """The timed FP32 solves (learned mode and plain block-Jacobi) against an
    FP64 solve of the same problem (the library's FP64 operator, block-Jacobi
    PCG to |r|^2/|b|^2 <= 1e-15), at the metric's stop (|r|/|b| <= 1e-6) and
    at tighter stops: per stop the solve's device time, its iterations and the
    largest relative RMS map error, so that the time each mode needs for maps
    within 1e-5 of the FP64 solve is on the record too."""
    t = time.time()
    m64 = sg.MapMaker(spec.ns, spec.nseg, spec.ndet, spec.nside, hwp=spec.hwp,
                      omega=prob["omega"], precision="f64", device=mm.device)
    m64.set_stream(stream.cuda_stream)
    m64.set_pointing(prob["ra"], prob["dec"], prob["psi"], dets, prob["isampmin"])
    for d in range(spec.ndet):
        m64.set_noise(d, prob["ispf"][d])
        m64.set_tod(d, prob["tod"][d])
    m64.rhs(chi2=False)
    r64 = m64.solve(precond="bj3", stop_crit=1e-15, maxiter=args.maxiter)
    x64 = m64.solution()
    m64.close()
    npix = mm.npix
    res = {"against": "FP64 solve of the same problem by the library's FP64 operator "
                      "(block-Jacobi PCG to |r|^2/|b|^2 <= 1e-15)",
           "fp64_iterations": r64["iterations"], "fp64_crit": r64["crit"],
           "fp64_seconds": time.time() - t, "bar": 1e-5}
    for pc in dict.fromkeys((precond, args.precond)):
        key = "learned" if pc == "learned" else pc
        sweep = []
        for stop in (STOP_CRIT, 1e-13, 1e-14):
            mm.rhs(chi2=False)
            rep = mm.solve(precond=pc, stop_crit=stop, maxiter=args.maxiter)
            errs = _map_errs(mm.solution(), x64, npix)
            worst = max(errs[k]["rms"] for k in "IQU")
            worst0 = max(errs[k]["rms_monopole_removed"] for k in "IQU")
            if stop == STOP_CRIT:
                res[key] = errs
            sweep.append({"stop_crit": stop, "iterations": rep["iterations"],
                          "converged": bool(rep["converged"]),
                          "solve_device_s": rep["device_seconds"], "max_rms": worst,
                          "max_rms_monopole_removed": worst0})
        res[key + "_by_stop"] = sweep
        ok = [r for r in sweep if r["converged"] and r["max_rms"] <= 1e-5]
        res[key + "_solve_s_to_1e-5_maps"] = ok[0]["solve_device_s"] if ok else None
    return res


def per_detector(sg, spec, prob, dets, stream, args):
    """The same workload through the per-detector operator (what detectors
    with distinct focal-plane offsets run): plain block-Jacobi solve time and
    the operator kernels' HBM throughput."""
    import torch
    os.environ["SANEPIC_GPU_GROUP_FILTER"] = "0"
    try:
        mp = sg.MapMaker(spec.ns, spec.nseg, spec.ndet, spec.nside, hwp=spec.hwp,
                         omega=prob["omega"], precision=spec.precision, device=torch.cuda.current_device())
        mp.set_stream(stream.cuda_stream)
        mp.set_pointing(prob["ra"], prob["dec"], prob["psi"], dets, prob["isampmin"])
    finally:
        os.environ.pop("SANEPIC_GPU_GROUP_FILTER", None)
    for d in range(spec.ndet):
        mp.set_noise(d, prob["ispf"][d])
        mp.set_tod(d, prob["tod"][d])
    assert not mp.group_mode()[0]
    for _ in range(2):
        mp.rhs(chi2=False)
        mp.solve(precond=args.precond, stop_crit=STOP_CRIT, maxiter=args.maxiter)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    ev0.record(stream)
    for _ in range(reps):
        mp.rhs(chi2=False)
        rep = mp.solve(precond=args.precond, stop_crit=STOP_CRIT, maxiter=args.maxiter)
    ev1.record(stream)
    torch.cuda.synchronize()
    sec = ev0.elapsed_time(ev1) / reps / 1e3
    prof = mp.profile_operator(reps=5)
    esz = 4 if spec.precision == "f32" else 8
    ns_all = spec.ndet * spec.nseg * spec.ns
    ng = mp.group_mode()[1] * spec.nseg * spec.ns
    npix = mp.npix
    m1 = spec.ns // 2 + 1
    kbytes = {"k_project": ng * (4 + 2 * esz) + ns_all * esz + npix * 4 * esz,
              "k_noise_filter": ns_all * 2 * esz + spec.ndet * m1 * esz,
              "k_detsum": ns_all * esz + ng * 4 * esz,
              "k_pt": ng * (4 + 2 * esz + 4 * esz) + npix * (3 * 8 + 8 + 4)}
    kms = {"k_project": prof["p_ms"], "k_noise_filter": prof["filter_ms"],
           "k_detsum": prof["detsum_ms"], "k_pt": prof["pt_ms"]}
    hbm, _ = peaks()
    mp.close()
    return {"operator": "per detector (SANEPIC_GPU_GROUP_FILTER=0)", "precond": args.precond,
            "seconds": sec, "iterations": rep["iterations"], "iter_per_sec": rep["iter_per_sec"],
            "kernels": {k: {"ms": kms[k], "GBps": kbytes[k] / (kms[k] * 1e-3) / 1e9,
                            "frac": kbytes[k] / (kms[k] * 1e-3) / 1e9 / hbm, "bytes": kbytes[k]}
                        for k in kbytes}}


def c3_block(sg, stream, args):
    """The largest single-GPU configuration (256 detectors, NSIDE 512, HWP,
    48 x 131,072 samples = 1.6e9 samples, FP32 operator), inputs resident:
    plain block-Jacobi PCG and the learned mode (coarse space trained on
    this workload and judged by plain PCG on a held-out problem), each from
    x0 = 0 to |r|/|b| <= 1e-6, with the learned solve's map error against an
    FP64 solve (the library's FP64 operator, block-Jacobi to 1e-15)."""
    import torch
    spec = synth.spec_from_name(C3)
    t0 = time.time()
    prob = synth.make_problem(spec)
    gen_s = time.time() - t0
    dets = sg.detectors_from_angles(prob["angles"])
    mm = sg.MapMaker(spec.ns, spec.nseg, spec.ndet, spec.nside, hwp=spec.hwp,
                     omega=prob["omega"], precision=spec.precision, device=torch.cuda.current_device())
    mm.set_stream(stream.cuda_stream)
    mm.set_pointing(prob["ra"], prob["dec"], prob["psi"], dets, prob["isampmin"])
    for d in range(spec.ndet):
        mm.set_noise(d, prob["ispf"][d])
        mm.set_tod(d, prob["tod"][d])
    tl = time.time()
    learn = mm.learn_train(npairs=args.learn_pairs, steps=-1, coarse_k=args.coarse_k,
                           coarse_vectors=args.coarse_vectors)
    learn_s = time.time() - tl
    res = {"workload": C3, "ndet": spec.ndet, "nside": spec.nside, "nseg": spec.nseg,
           "ns": spec.ns, "hwp": True, "samples": spec.ndet * spec.nseg * spec.ns,
           "npix_obs": mm.npix, "generation_s": gen_s, "learn_s": learn_s,
           "learned_part": {0: "none: plain block-Jacobi PCG", 1: "patch network",
                            2: "coarse space"}[learn["kind"]],
           "validation": {"plain_iterations": learn["val_plain_iters"],
                          "coarse_iterations": learn["val_coarse_iters"],
                          "plain_ms": learn["val_plain_ms"], "coarse_ms": learn["val_coarse_ms"]},
           "coarse_vectors": learn.get("coarse_k")}
    sols = {}
    for pc in ("bj3", "learned"):
        for _ in range(2):
            mm.rhs(chi2=False)
            mm.solve(precond=pc, stop_crit=STOP_CRIT, maxiter=args.maxiter)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 3
        ev0.record(stream)
        for _ in range(reps):
            mm.rhs(chi2=False)
            rep = mm.solve(precond=pc, stop_crit=STOP_CRIT, maxiter=args.maxiter)
        ev1.record(stream)
        torch.cuda.synchronize()
        res["plain" if pc == "bj3" else "learned"] = {
            "seconds": ev0.elapsed_time(ev1) / reps / 1e3, "iterations": rep["iterations"],
            "converged": bool(rep["converged"])}
        sols[pc] = mm.solution()
    prof = mm.profile_operator(reps=5)
    res["operator_ms"] = prof
    npix = mm.npix
    mm.close()
    m64 = sg.MapMaker(spec.ns, spec.nseg, spec.ndet, spec.nside, hwp=spec.hwp,
                      omega=prob["omega"], precision="f64", device=torch.cuda.current_device())
    m64.set_stream(stream.cuda_stream)
    m64.set_pointing(prob["ra"], prob["dec"], prob["psi"], dets, prob["isampmin"])
    for d in range(spec.ndet):
        m64.set_noise(d, prob["ispf"][d])
        m64.set_tod(d, prob["tod"][d])
    m64.rhs(chi2=False)
    r64 = m64.solve(precond="bj3", stop_crit=1e-15, maxiter=args.maxiter)
    x64 = m64.solution()
    m64.close()
    res["map_error"] = {"against": "library FP64 operator, block-Jacobi PCG to 1e-15",
                        "fp64_iterations": r64["iterations"],
                        "plain": _map_errs(sols["bj3"], x64, npix),
                        "learned": _map_errs(sols["learned"], x64, npix)}
    return res


def mlp_gemm_roofline(sg, mm):
    """Tensor-core throughput of the network's GEMM (tcgen05, BF16 in, FP32
    accumulate) on the inference shape of this workload and a large training
    shape, CUDA-event timed, against the measured BF16 peak."""
    peak, kind = bf16_peak()

    def bf16_bits(a):  # round to nearest even, upper 16 bits of FP32
        u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
        return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)

    rows = -(-mm.npix // 256)
    rows = max(128, -(-rows // 128) * 128)
    out = {"peak_tflops": peak, "peak_kind": kind, "shapes": []}
    rng = np.random.default_rng(0)
    for M, N, K in ((rows, 256, 768), (8192, 768, 8192)):
        A = bf16_bits(rng.standard_normal((M, K)))
        B = bf16_bits(rng.standard_normal((N, K)))
        _, ms = sg.gemm_bf16(A, B, reps=20)
        tf = 2.0 * M * N * K / (ms * 1e-3) / 1e12
        out["shapes"].append({"M": M, "N": N, "K": K, "ms": ms, "tflops": tf,
                              "frac": tf / peak})
    return out


def run_batch(args):
    """32 uneven independent problems (synth.batch_specs): every problem's
    operator autotuned, then all solved together (sg_solve_batch: one CUDA
    stream and captured iteration graphs per problem) and, for comparison,
    one after another.  value = time until every problem reaches
    |r|/|b| <= 1e-6 (or the iteration cap) in the learned mode, each problem
    with the coarse space built from its own plain solves where plain PCG
    judged it faster; the plain batch time, per-problem iterations and device
    times are reported beside it."""
    import torch

    import sanepic_gb300 as sg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    specs = synth.batch_specs(32)
    t0 = time.time()
    makers = []
    for sp in specs:
        prob = synth.make_problem(sp)
        mm = sg.from_problem(prob, precision="f32", device=local)
        # one-detector problems leave most Q/U blocks nearly singular: mask
        # those (sg_set_pol_rcond) so that every problem is well posed
        mm.set_pol_rcond(args.pol_rcond)
        mm.rhs()
        makers.append(mm)
        del prob
    gen_s = time.time() - t0
    tunes = [mm.autotune() for mm in makers]
    # the learned mode: each problem builds its own coarse space from its own
    # plain solves (the coarse space belongs to the operator) and plain PCG
    # judges it on a held-out sky; the patch network, which never wins that
    # judgement, is not trained here
    learn = None
    if not args.no_learn:
        tl = time.time()
        learn = [mm.learn_train(npairs=256, steps=-1, coarse_k=args.coarse_k,
                                coarse_vectors=args.coarse_vectors) for mm in makers]
        for mm in makers:
            mm.rhs()
        learn_s = time.time() - tl

    def batch(precond):
        torch.cuda.synchronize()
        t = time.perf_counter()
        reps = sg.solve_batch(makers, precond=precond, stop_crit=STOP_CRIT, maxiter=args.maxiter)
        torch.cuda.synchronize()
        return time.perf_counter() - t, reps

    for _ in range(args.warmup):
        batch(args.precond)
    times, reps = [], None
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t, reps = batch(args.precond)
            times.append(t)
    clocks = clk.summary()
    value = float(np.median(times))
    # one after another (each solve alone on the GPU)
    torch.cuda.synchronize()
    t = time.perf_counter()
    seq = [mm.solve(precond=args.precond, stop_crit=STOP_CRIT, maxiter=args.maxiter)
           for mm in makers]
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t
    learned = None
    plain_value = value
    if learn is not None:
        # the value is the learned mode's batch time, the plain one is kept beside it
        batch("learned")
        ltimes, lreps = [], None
        with ClockSampler(local) as clk:
            for _ in range(args.steps):
                lt, lreps = batch("learned")
                ltimes.append(lt)
        clocks = clk.summary()
        value = float(np.median(ltimes))
        learned = {"batch_s": value, "plain_batch_s": plain_value, "training_s": learn_s,
                   "coarse_space_used": sum(1 for r in learn if r["kind"] == 2),
                   "problems": [{"iterations": q["iterations"], "converged": bool(q["converged"]),
                                 "device_s": q["device_seconds"], "coarse_k": r["coarse_k"],
                                 "used": r["kind"] == 2,
                                 "val_plain_iterations": r["val_plain_iters"],
                                 "val_coarse_iterations": r["val_coarse_iters"]}
                                for q, r in zip(lreps, learn)]}
    samples = sum(sp.ndet * sp.nseg * sp.ns for sp in specs)
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scan, iid sky, 1/f noise), 32 uneven problems",
        "config": {"workload": "batch32_uneven", "problems": len(specs), "samples": samples,
                   "precond": "learned (per-problem coarse space, judged by block-Jacobi PCG)"
                   if learn is not None else args.precond, "stop": "|r|/|b| <= 1e-6",
                   "solve": "concurrent: one stream + captured graphs per problem",
                   "pol_rcond": args.pol_rcond},
        "sequential_s": seq_s,
        "problems": [{"name": sp.name, "iterations": r["iterations"],
                      "device_s": r["device_seconds"], "converged": bool(r["converged"]),
                      "alone_s": q["device_seconds"], "cluster_size": tu["cluster_size"],
                      "pt_lanes": tu["pt_lanes"]}
                     for sp, r, q, tu in zip(specs, reps, seq, tunes)],
        "gpu_launches": int(sum(r["kernel_launches"] for r in reps)),
        "clocks": clocks, "generation_s": gen_s,
    }
    if learned is not None:
        line["learned"] = learned
    if rank == 0:
        print(json.dumps(line), flush=True)
    for mm in makers:
        mm.close()


# ---------------------------------------------------------------------------
# The threaded port of the reference's path (oracle/cgpar.c) against the
# shimmed reference itself on the same workload and cores (x86, 8 cores; the
# reference cannot be built on the GPU host): the port's RHS-to-1e-6 interval
# takes PORT_OVER_REFERENCE of the reference's (oracle/calibrate_port.py,
# profiles/cpu_port_vs_reference.md).
PORT_OVER_REFERENCE = {"c2_64det_nside256": 0.82, "c1_4det_nside64": 0.52}


def port_solve(spec, nthreads, maxiter):
    """One whole run of the reference's path on the host: the threaded port
    (setup, RHS, the reference's diagonal preconditioner, PCG to
    |r|/|b| <= 1e-6), its phase times in seconds."""
    import oracle  # the CPU checker; only the CPU-baseline legs of bench.py use it
    prob = synth.make_problem(spec)
    t = time.time()
    r = oracle.cpu_solve(prob, nthreads, stop_crit=STOP_CRIT, maxiter=maxiter)
    r["wall_s"] = time.time() - t
    return r


def reference_cpu(args, spec):
    """CPU baseline beside the GPU line: the threaded port on every host
    core, timed on a bounded sample of the workload -- the same scan, sizes
    and noise model with 8 of the detectors, solved from scratch to
    |r|/|b| <= 1e-6 -- and scaled to the workload's detector count (the
    per-iteration work is linear in detectors; the iterations are the
    sample's).  The whole workload is timed by --impl reference."""
    import dataclasses
    cores = os.cpu_count() or 2
    nd = min(8, spec.ndet)
    sp = dataclasses.replace(spec, ndet=nd, name=spec.name + f"_sample{nd}det")
    r = port_solve(sp, cores, args.maxiter)
    t = r["times"]["to_stop"]
    scale = spec.ndet / nd
    return {"value": t * scale if t > 0 else None, "unit": "s", "cores": cores, "kind": "port",
            "sample": (f"{nd} of {spec.ndet} detectors, every segment ({nd * spec.nseg} x "
                       f"{spec.ns} samples): RHS + diagonal preconditioner + PCG to |r|/|b| <= "
                       f"1e-6 measured ({t:.2f} s, {r['iterations']} iterations), x{scale:g} "
                       "detectors"),
            "sample_phases_s": r["times"], "sample_iterations": r["iterations"]}


def run_reference(args):
    """--impl reference: the reference's path on the host cores for the whole
    workload -- the threaded port of sanepic.cc's algorithm (oracle/cgpar.c)
    in its parallel layout, every host thread, each run from scratch (value =
    RHS + diagonal preconditioner + PCG until |r|/|b| <= 1e-6, the scope of
    the GPU value plus the reference's preconditioner build).  A run takes
    about two minutes, so `steps` reports the runs actually made within the
    time budget, not the requested count."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    spec = synth.spec_from_name(args.config)
    cores = os.cpu_count() or 2
    runs = []
    t0 = time.time()
    while len(runs) < max(1, args.steps):
        runs.append(port_solve(spec, cores, args.maxiter))
        per = (time.time() - t0) / len(runs)
        if time.time() - t0 + per > args.ref_budget_s:
            break
    vals = sorted(r["times"]["to_stop"] for r in runs if r["times"]["to_stop"] > 0)
    value = vals[len(vals) // 2] if vals else None
    last = runs[-1]
    cb = {"value": value, "unit": "s", "cores": cores, "kind": "port",
          "sample": (f"the whole workload ({spec.ndet} det x {spec.nseg} x {spec.ns} samples), "
                     f"{len(runs)} run(s) from scratch; timed: RHS + the reference's diagonal "
                     "preconditioner + PCG to |r|/|b| <= 1e-6"),
          "phases_s": last["times"], "iterations": last["iterations"],
          "run_wall_s": [r["wall_s"] for r in runs],
          "port_over_reference": PORT_OVER_REFERENCE.get(args.config),
          "calibration": "oracle/calibrate_port.py: the shimmed reference and this port on the "
                         "same workload and cores (x86); the reference cannot be built here"}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s",
            "n_gpus": world, "steps": len(runs), "warmup": 0,
            "requested": {"steps": args.steps, "warmup": args.warmup},
            "ms_per_step": value * 1e3 if value else None,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded spin+precession scan, iid sky, 1/f noise)",
            "config": {"workload": args.config, "ndet": spec.ndet, "nside": spec.nside,
                       "nseg": spec.nseg, "ns": spec.ns, "precond": "diag (the reference's)",
                       "stop": "|r|/|b| <= 1e-6"},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if value is None:
        line["unavailable"] = "the port did not reach |r|/|b| <= 1e-6"
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2_64det_nside256")
    ap.add_argument("--precond", default="bj3")
    ap.add_argument("--maxiter", type=int, default=2000)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--compare-diag", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-budget-s", type=float, default=240.0,
                    help="--impl reference: no new run starts past this many seconds")
    ap.add_argument("--no-learn", action="store_true")
    ap.add_argument("--learn-pairs", type=int, default=512)
    ap.add_argument("--learn-steps", type=int, default=1500)
    ap.add_argument("--coarse-k", type=int, default=0)
    ap.add_argument("--coarse-vectors", type=int, default=0)
    ap.add_argument("--no-map-error", action="store_true")
    ap.add_argument("--pol-rcond", type=float, default=1e-3,
                    help="batch32: mask Q/U of pixels whose 3x3 hit block is this ill-conditioned")
    ap.add_argument("--no-per-detector", action="store_true")
    ap.add_argument("--c3", type=int, default=1, help="add the C3 block (1) or not (0)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "batch32":
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
