"""Times the reference built against the project's shims (oracle/_ref/sanepic)
and the threaded port of its path (cgpar.c, what bench.py's CPU baseline runs
on the GPU host) on the same workload and the same host cores, and prints one
JSON line: the port's time relative to the reference's.

The reference's source does not travel to the GPU host and no aarch64 build
of it exists there, so this calibration runs where the reference was built:
    make -C oracle ref REFERENCE_SRC=<reference checkout>/src/sanepic.cc
    python oracle/calibrate_port.py --config c2_64det_nside256 --procs 8

Reference timing follows its own printed lines, read as they arrive
(stdbuf -oL): from "PtNd Computed..." (sanepic.cc:1131-1132, after the
right-hand side) to the first "iter = .., crit = .." line with
crit <= 1e-12 (|r|/|b| <= 1e-6, sanepic.cc:1607-1609), plus its whole wall
time.  The port's matching interval is its precond + solve phases up to
crit <= 1e-12 (cgpar.c's to_stop minus rhs).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sanepic_gb300 import synth  # noqa: E402


def time_reference(prob, procs, stop=1e-12):
    exe = os.path.join(HERE, "_ref", "sanepic")
    with tempfile.TemporaryDirectory() as td:
        args = synth.write_reference_tree(prob, td)
        env = dict(os.environ, SHIM_MPI_NP=str(procs))
        t0 = time.time()
        p = subprocess.Popen(["stdbuf", "-oL", exe] + args, env=env, stdout=subprocess.PIPE,
                             stderr=subprocess.DEVNULL, text=True)
        t_ptnd = t_stop = None
        iters, first_stop_iter = [], None
        for line in p.stdout:
            now = time.time()
            if t_ptnd is None and line.startswith("PtNd Computed"):
                t_ptnd = now
            m = re.match(r"iter = (\d+), crit = ([^,\s]+)", line)
            if m:
                iters.append((int(m.group(1)), float(m.group(2)), now))
                if t_stop is None and float(m.group(2)) <= stop:
                    t_stop, first_stop_iter = now, int(m.group(1))
        p.wait()
        wall = time.time() - t0
    rate = None
    if len(iters) > 2:
        rate = (len(iters) - 1) / (iters[-1][2] - iters[0][2])
    return {"rc": p.returncode, "wall_s": wall,
            "ptnd_to_1e-12_s": (t_stop - t_ptnd) if (t_stop and t_ptnd) else None,
            "iterations_to_1e-12": None if first_stop_iter is None else first_stop_iter + 1,
            "iterations_total": len(iters), "iter_per_s": rate}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2_64det_nside256")
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 2,
                    help="reference ranks (1 master + procs-1 workers); the port uses procs-1 threads")
    a = ap.parse_args()
    spec = synth.spec_from_name(a.config)
    prob = synth.make_problem(spec)
    ref = time_reference(prob, a.procs)
    t = time.time()
    port = oracle.cpu_solve(prob, max(1, a.procs - 1), stop_crit=1e-12)
    port_wall = time.time() - t
    tt = port["times"]
    port_interval = tt["to_stop"] - tt["rhs"] if tt["to_stop"] > 0 else None
    out = {"config": a.config, "host_cores": os.cpu_count(), "reference_procs": a.procs,
           "port_threads": max(1, a.procs - 1), "reference": ref,
           "port": {"wall_s": port_wall, "phases_s": tt, "iterations": port["iterations"],
                    "ptnd_to_1e-12_s": port_interval},
           "port_over_reference": (port_interval / ref["ptnd_to_1e-12_s"])
           if (port_interval and ref["ptnd_to_1e-12_s"]) else None,
           "fft": "both use oracle/fft64.c (the reference through the project's FFTW shim)"}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
