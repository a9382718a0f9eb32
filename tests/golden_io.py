"""Loader for the golden vectors in tests/golden/*.npz."""
import glob
import json
import os

import numpy as np

from fiesta_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))


class Case:
    def __init__(self, path):
        z = np.load(path)
        self.meta = json.loads(str(z["meta"]))
        self.name = self.meta["name"]
        self.cfg = abi.config_from_dict(self.meta["config"])
        self.steps = int(self.meta["steps"])
        self.U0 = np.asfortranarray(z["U0"])
        self.R1 = np.asfortranarray(z["R1"])
        self.UN = np.asfortranarray(z["UN"])
        self.SN = np.asfortranarray(z["SN"])


def load_all():
    return [Case(p) for p in sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))]


def same(a, b):
    """IEEE equality of every element (so +0 == -0), NaN matching NaN."""
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def rel_l2(a, b, interior=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    num = np.linalg.norm((a - b).ravel())
    den = np.linalg.norm(b.ravel())
    return num / den if den > 0 else num


def interior(cfg, A):
    ng = cfg.ng
    if cfg.ndim == 3:
        return A[ng:-ng, ng:-ng, ng:-ng]
    return A[ng:-ng, ng:-ng]
