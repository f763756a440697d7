"""Loader of the committed golden vectors (tests/golden/*.npz, produced by
tests/golden/make_golden.py from the reference's own solver classes)."""
import glob
import json
import os

import numpy as np

from hydro_gb300 import capi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        n = os.path.splitext(os.path.basename(p))[0]
        if n != "cavity_sample" and not n.startswith("vts"):  # solver runs only
            out.append(n)
    return out


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = {k: z[k] for k in z.files}
    g["desc"] = capi.desc_from_dict(json.loads(str(z["desc"])))
    g["nsteps"] = int(z["nsteps"])
    g["gpu_comparable"] = bool(z["gpu_comparable"])
    g["heat"] = capi.heat_from_dict(json.loads(str(z["heat"]))) if "heat" in z.files else None
    return g


def sample():
    z = np.load(os.path.join(GOLDEN, "cavity_sample.npz"))
    return {k: z[k] for k in z.files}
