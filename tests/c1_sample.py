"""Class-stratified selections from the committed c1 quartet list (tests/golden/c1_quartets.npz)."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def c1_quartets():
    return np.load(os.path.join(HERE, 'golden', 'c1_quartets.npz'))['quartets']


def kernel_class(mol, qs):
    """(li, lj, lk, ll) of each quartet in the kernels' order: larger l first inside each pair,
    then the pair with the larger (l_first, l_second) first."""
    L = mol.bas[:, 1][np.asarray(qs)]
    a = np.maximum(L[:, 0], L[:, 1]); b = np.minimum(L[:, 0], L[:, 1])
    c = np.maximum(L[:, 2], L[:, 3]); d = np.minimum(L[:, 2], L[:, 3])
    swap = (a * 16 + b) < (c * 16 + d)
    return np.where(swap[:, None], np.stack([c, d, a, b], 1), np.stack([a, b, c, d], 1))


def stratified(mol, qs, per_class):
    """The first per_class quartets (list order) of every kernel class; returns (quartets,
    class tuples)."""
    k = kernel_class(mol, qs)
    key = ((k[:, 0] * 8 + k[:, 1]) * 8 + k[:, 2]) * 8 + k[:, 3]
    keep = []
    for u in np.unique(key):
        keep.extend(np.nonzero(key == u)[0][:per_class].tolist())
    keep = np.sort(np.array(keep, dtype=np.int64))
    return np.ascontiguousarray(qs[keep]), k[keep]
