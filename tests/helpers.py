"""Shared helpers for the test suite (fixture loading, key alignment)."""
import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def align(level_ref, suppt_ref, level, suppt):
    """Permutation p with (level_ref[p], suppt_ref[p]) == (level, suppt) row by row."""
    idx = {tuple(a) + tuple(b): i for i, (a, b) in enumerate(zip(level_ref, suppt_ref))}
    perm = np.array([idx[tuple(a) + tuple(b)] for a, b in zip(level, suppt)])
    assert len(perm) == len(idx), "element sets differ"
    return perm


def ic_terms(ic, dim):
    import amdg_oracle as O
    if ic == "sin_sum":
        return O.sin_sum_terms(dim)
    if ic == "sin_prod":
        return [lambda x, d: math.sin(2 * math.pi * x)]
    raise ValueError(ic)


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))
