"""Shared helpers for the tests (fixture loading, error metrics)."""
import os

import numpy as np

from itn_gb300 import graphs as G

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name)))
    g = G.Graph(int(len(d["off"]) - 1), d["off"], d["nbr"], d["bond"], d["rev"], d["phys"],
                int(d["layers"]))
    return g, d


def max_rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def msg_rel(g, a, b):
    """Largest per-message relative error (each message measured in its own scale)."""
    worst = 0.0
    for s in range(g.nslots):
        x = a[g.moff[s]:g.moff[s + 1]]
        y = b[g.moff[s]:g.moff[s + 1]]
        worst = max(worst, float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300)))
    return worst
