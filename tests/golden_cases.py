"""Loader for the golden fixtures written by tests/golden/make_golden.py."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# calcqpi cases; the mkwf_* directories hold the orbital-file tool's cases and the bs_* ones the
# band-structure histograms (own test files)
NAMES = sorted(d for d in os.listdir(GOLDEN)
               if os.path.isdir(os.path.join(GOLDEN, d)) and not d.startswith(("_", "mkwf_", "bs_")))


def load(name):
    d = os.path.join(GOLDEN, name)
    with open(os.path.join(d, "meta.json")) as fh:
        meta = json.load(fh)
    z = np.load(os.path.join(d, "ref_ldos64.npz"))
    return d, meta, {k: z[k] for k in z.files}


def energies(meta):
    lo, hi = meta["energies"]
    L = meta["layers"]
    if L == 1:
        return np.array([lo])
    return np.array([(hi - lo) * k / (L - 1.0) + lo for k in range(L)])


def josephson(meta):
    """(deltat, etat) of a josephson-mode case with the driver's defaults (deltat 0.001,
    etat = eta; src/calcqpi.cc:137,249-251), or None for a wannier-mode case."""
    j = meta.get("josephson")
    if not j:
        return None
    return (0.001 if j[0] is None else j[0], meta["eta"] if j[1] is None else j[1])


def uspf_pos(meta):
    """Band positions of an output=uspf case, (0, 0) where pos[i] is not given."""
    if meta.get("output") != "uspf":
        return None
    return [tuple(meta.get("pos", {}).get(str(i), (0.0, 0.0)))[:2] for i in range(meta["maxband"])]


def uspf_pre(meta):
    if meta.get("output") != "uspf":
        return None
    pre = list(meta.get("prearr", ()))[:meta["maxband"]]
    return pre + [1.0] * (meta["maxband"] - len(pre))
