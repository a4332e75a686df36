"""Generate tests/golden/c1_schwarz.npz: libcint's Schwarz decisions on a sample of c1 quartets.

Run where libcint's sources exist (oracle/Makefile builds oracle/_ref/libcint.so from them):
    make -C oracle ref && python tests/golden/make_schwarz_sample.py

c1 = libcint_gb300.molecules.config1(seed=0).  20000 unique quartets (i>=j, k>=l, ij>=kl) are drawn
uniformly (seed 1), every shell pair they touch gets Q_ij = sqrt(max |(ij|ij)|) from libcint's own
int2e_sph (the definition tests/golden/make_c1_sample.py screens the benchmark list with), and the
file records the pairs, their Q, the quartets and libcint's decision Q_ij Q_kl >= 1e-12 for each.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libcint_gb300 import molecules as M  # noqa: E402

N = 20000


def main():
    mol = M.config1(seed=0)
    lib = ctypes.CDLL(os.path.join(ROOT, 'oracle', '_ref', 'libcint.so'))
    lib.int2e_sph.restype = ctypes.c_int
    ii, jj = np.tril_indices(mol.nbas)
    pairs = np.stack([ii, jj], 1).astype(np.int32)
    rng = np.random.RandomState(1)
    a = rng.randint(0, len(pairs), 2 * N)
    b = rng.randint(0, len(pairs), 2 * N)
    keep = b <= a
    a, b = a[keep][:N], b[keep][:N]
    used = np.unique(np.concatenate([a, b]))
    P = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    Q = np.zeros(len(used))
    for t, p in enumerate(used):
        i, j = int(pairs[p, 0]), int(pairs[p, 1])
        n = mol.nsph(i) * mol.nsph(j)
        buf = np.zeros(n * n)
        shls = np.array([i, j, i, j], np.int32)
        lib.int2e_sph(P(buf), None, P(shls), P(mol.atm), mol.natm, P(mol.bas), mol.nbas,
                      P(mol.env), None, None)
        Q[t] = np.sqrt(np.abs(buf).max())
    pos = {int(p): t for t, p in enumerate(used)}
    qa = Q[[pos[int(x)] for x in a]]
    qb = Q[[pos[int(x)] for x in b]]
    quartets = np.concatenate([pairs[a], pairs[b]], 1).astype(np.int32)
    keep = qa * qb >= 1e-12
    np.savez_compressed(os.path.join(HERE, 'c1_schwarz.npz'), pairs=pairs[used], q=Q,
                        quartets=quartets, keep=keep,
                        note=np.array('c1 seed 0; quartet sample seed 1; Q and decisions by libcint'))
    print('pairs', len(used), 'quartets', len(quartets), 'kept', int(keep.sum()))


if __name__ == '__main__':
    main()
