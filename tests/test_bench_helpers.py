"""The host-side helpers bench.py uses to train the batched solves' classifier: the features match
the feature kernel's definition (log10(|c| + 1e-20)/20 + 1 of the element's block, then of its
parent and grandparent along each dimension, 0 where absent) and the labels the criterion's
choice (block norm above eps)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


class FakeGrid:
    """Element set given by packed 1D orders (nmax bits per dimension, dimension 0 highest)."""

    def __init__(self, dim, nmax, keys, seed=0):
        self.dim, self.nmax, self.block = dim, nmax, 3 ** dim
        self.keys = np.sort(np.asarray(keys, np.int64))
        self.num_elements = len(self.keys)
        self.u = np.random.default_rng(seed).standard_normal((self.num_elements, self.block))
        self.u[::3] *= 1e-8

    def elements(self):
        m = (1 << self.nmax) - 1
        o = np.stack([(self.keys >> (self.nmax * (self.dim - 1 - d))) & m for d in range(self.dim)], 1)
        lv = np.where(o == 0, 0, np.floor(np.log2(np.maximum(o, 1))).astype(int) + 1)
        sp = np.where(o == 0, 1, 2 * (o - (1 << np.maximum(lv - 1, 0))) + 1)
        return lv, sp

    def coefficients(self):
        return self.u


def sparse_keys(dim, nmax, total):
    orders = range(1 << nmax)
    out = [0]
    for d in range(dim):
        out = [(k << nmax) | o for k in out for o in orders]
    return [k for k in out if sum(((k >> (nmax * (dim - 1 - d))) & ((1 << nmax) - 1)).bit_length()
                                  for d in range(dim)) <= total]


def test_grid_features_match_the_feature_kernel_definition():
    dim, nmax = 2, 3
    keys = sparse_keys(dim, nmax, 3)
    keys.remove((2 << nmax) | 0)  # a hole: some elements lose their parent
    g = FakeGrid(dim, nmax, keys)
    assert np.array_equal(bench.element_keys(g), g.keys)
    F = bench.grid_features(g)
    B = g.block
    mag = (np.log10(np.abs(g.u) + 1e-20) / 20.0 + 1.0).astype(np.float32)
    index = {int(k): i for i, k in enumerate(g.keys)}
    mask = (1 << nmax) - 1
    assert np.array_equal(F[:, :B], mag)
    for e, key in enumerate(g.keys):
        for d in range(dim):
            shift = nmax * (dim - 1 - d)
            k, alive = int(key), True
            for gen in range(2):
                o = (k >> shift) & mask
                alive = alive and o > 0
                k = (k & ~(mask << shift)) | ((0 if o == 1 else o // 2) << shift)
                j = index.get(k, -1) if alive else -1
                want = mag[j] if j >= 0 else np.zeros(B, np.float32)
                slot = 1 + 2 * d + gen
                assert np.array_equal(F[e, slot * B:(slot + 1) * B], want), (e, d, gen)


def test_refine_labels_are_the_criterion():
    g = FakeGrid(2, 3, sparse_keys(2, 3, 3), seed=1)
    lab = bench.refine_labels(g, 1e-3)
    norms = np.sqrt(np.sum(g.u ** 2, axis=1))
    assert np.array_equal(lab, np.where(norms > 1e-3, 0, 1))
    assert set(lab.tolist()) == {0, 1}
