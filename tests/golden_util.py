"""Helpers to load the golden fixtures made from the reference PySPH."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as d:
        return {k: d[k] for k in d.files}


def inputs(g, array):
    pre = "in_%s_" % array
    return {k[len(pre):]: v for k, v in g.items() if k.startswith(pre)}


def csr_sets(offsets, index):
    return [set(index[offsets[i]:offsets[i + 1]].tolist()) for i in range(len(offsets) - 1)]


def normwise(a, ref):
    """max |a - ref| / max |ref| (the per-field parity metric)."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref).max()
    if scale == 0:
        return float(np.abs(a).max())
    return float(np.abs(a - ref).max() / scale)
