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


def rel_percentiles(a, ref, floor=1e-3):
    """Per-particle relative error |a - ref| / |ref| over the particles with
    |ref| above floor * max |ref|: (p50, p99, max, particles counted)."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref).max()
    keep = np.abs(ref) > floor * scale
    if not keep.any():
        return 0.0, 0.0, 0.0, 0
    r = np.abs(a[keep] - ref[keep]) / np.abs(ref[keep])
    return float(np.percentile(r, 50)), float(np.percentile(r, 99)), float(r.max()), int(keep.sum())
