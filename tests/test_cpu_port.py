"""The CPU baseline's multi-threaded run of the reference's path (oracle
cgpar.c, what bench.py times) against the single-threaded oracle and the
reference's own outputs: same iterations, same maps."""
import numpy as np

import oracle
from golden_util import load_log, load_outputs, load_problem
from sanepic_gb300 import synth


def test_threaded_port_matches_single_thread_oracle():
    for hwp in (False, True):
        spec = synth.ProblemSpec("t", ndet=3, nside=16, nseg=6, ns=2048, hwp=hwp, fknee=0.05,
                                 problem=13)
        prob = synth.make_problem(spec)
        out, meta = oracle.run_pipeline(prob, precond="diag", stop_crit=1e-12, maxiter=500)
        for nthreads in (1, 4):
            r = oracle.cpu_solve(prob, nthreads, stop_crit=1e-12, maxiter=500)
            assert r["npix"] == meta["npix"]
            assert abs(r["iterations"] - meta["iters"]) <= 1
            x = meta["setup"].expand  # compact -> full, for the comparison below
            npix = r["npix"]
            for c, k in enumerate("IQU"):
                got = x(r["x"][c * npix:(c + 1) * npix])
                np.testing.assert_allclose(got, out[k], rtol=0, atol=1e-9 * np.abs(out[k]).max())
            assert r["times"]["to_stop"] > 0


def test_threaded_port_reproduces_reference_log():
    name = "golden_4det_nside16"
    prob = load_problem(name)
    log = load_log(name)
    r = oracle.cpu_solve(prob, 3, stop_crit=1e-15, maxiter=2000)
    ref_crit = np.array([c[1] for c in log["crit"]])
    n = min(10, len(ref_crit))
    np.testing.assert_allclose(r["crit"][:n], ref_crit[:n], rtol=1e-6)
    assert abs(r["iterations"] - log["iterations"]) <= 2
    ref = load_outputs(name)
    s = oracle.Setup(prob)
    npix = r["npix"]
    for c, k in enumerate("IQU"):
        got = s.expand(r["x"][c * npix:(c + 1) * npix])
        d = got - ref[k]
        if k == "I":
            obs = ref[k] != 0
            d = (d - d[obs].mean()) * obs
        assert np.sqrt(np.mean(d ** 2)) < 1e-6 * np.sqrt(np.mean(ref[k] ** 2)), k
