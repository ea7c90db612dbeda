"""Helpers to read the golden fixtures of tests/golden (written by tests/golden/make_golden.py)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def cores(z, prefix):
    key = prefix + "_n"
    if key not in z:
        return None
    return [z["%s_%d" % (prefix, i)] for i in range(int(z[key]))]


def params(z):
    return {k[2:]: z[k].item() for k in z.files if k.startswith("p_")}


def solve_fixtures():
    return sorted(f for f in os.listdir(GOLDEN) if f.startswith("solve_") and f.endswith(".npz"))
