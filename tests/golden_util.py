"""Loading the reference-generated fixtures under tests/golden/."""
import json
import os

import numpy as np

from sanepic_gb300 import synth

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["golden_4det_nside16", "golden_2det_nside16_hwp"]


def load_problem(name):
    z = np.load(os.path.join(GOLDEN_DIR, f"{name}_inputs.npz"))
    ndet, nside, nseg, ns, hwp = (int(v) for v in z["dims"])
    spec = synth.ProblemSpec(name, ndet=ndet, nside=nside, nseg=nseg, ns=ns, hwp=bool(hwp))
    return dict(spec=spec, ra=z["ra"], dec=z["dec"], psi=z["psi"],
                isampmin=z["isampmin"], angles=z["angles"], omega=float(z["omega"]),
                ispf=z["ispf"], tod=z["tod"], names=[str(n) for n in z["names"]])


def load_outputs(name):
    z = np.load(os.path.join(GOLDEN_DIR, f"{name}_ref_outputs.npz"))
    return {k: z[k] for k in z.files}


def load_log(name):
    with open(os.path.join(GOLDEN_DIR, f"{name}_ref_log.json")) as f:
        return json.load(f)


def rel_rms(a, b, remove_monopole=False):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    ref = np.asarray(b, np.float64)
    if remove_monopole:
        obs = ref != 0
        d = d - d[obs].mean() * obs
    den = np.sqrt(np.mean(ref ** 2))
    return float(np.sqrt(np.mean(d ** 2)) / den) if den > 0 else float(np.sqrt(np.mean(d ** 2)))
