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


def is_sampled(z):
    """A fixture that summarises the reference's solution by sampled entries (large workloads)."""
    return "sample_x" in z.files


def solve_fixtures(kind="all", max_cpp_s=None):
    """Whole-solve fixtures: ``kind`` "full" (the reference's solution cores stored), "sampled"
    (its solution summarised by sampled entries, norm, ranks and residual) or "all"; with
    ``max_cpp_s`` only those whose reference solve took at most that many seconds."""
    out = []
    for f in sorted(os.listdir(GOLDEN)):
        if not (f.startswith("solve_") and f.endswith(".npz")):
            continue
        z = load(f)
        sampled = is_sampled(z)
        if kind == "full" and sampled or kind == "sampled" and not sampled:
            continue
        if max_cpp_s is not None and float(z["t_cpp"]) > max_cpp_s:
            continue
        out.append(f)
    return out
