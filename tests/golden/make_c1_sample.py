"""Generate tests/golden/c1_quartets.npz: the Schwarz-screened quartet sample of the c1 workload.

Run where libcint's sources exist (oracle/Makefile builds oracle/_ref/libcint.so from them):
    make -C oracle ref && python tests/golden/make_c1_sample.py

c1 = libcint_gb300.molecules.config1(seed=0).  Unique quartets (i>=j, k>=l, ij>=kl) are drawn
uniformly (seed 0) and kept when Q_ij * Q_kl >= 1e-12, Q_ij = sqrt(max |(ij|ij)|) computed by
libcint's own int2e_sph, until N = 100000 survive.  The GPU benchmark and the CPU baseline both
evaluate exactly this list, so the surviving quartet list is identical by construction.
"""
import ctypes
import os
import sys
from multiprocessing import Pool

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libcint_gb300 import molecules as M  # noqa: E402

N = 100000
SEED = 0
_mol = None
_lib = None


def _init():
    global _mol, _lib
    _mol = M.config1(seed=0)
    _lib = ctypes.CDLL(os.path.join(ROOT, 'oracle', '_ref', 'libcint.so'))
    _lib.int2e_sph.restype = ctypes.c_int


def _q(pair):
    i, j = int(pair[0]), int(pair[1])
    mol = _mol
    n = mol.nsph(i) * mol.nsph(j)
    buf = np.zeros(n * n)
    shls = (ctypes.c_int * 4)(i, j, i, j)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    _lib.int2e_sph(P(buf), None, shls, P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env),
                   None, None)
    return float(np.sqrt(np.abs(buf).max()))


def main():
    mol = M.config1(seed=0)
    ii, jj = np.tril_indices(mol.nbas)
    pairs = np.stack([ii, jj], 1).astype(np.int32)
    npair = len(pairs)
    rng = np.random.RandomState(SEED)
    Q = np.full(npair, -1.0)
    out = []
    need = N
    with Pool(os.cpu_count(), initializer=_init) as pool:
        while need > 0:
            m = max(4 * need, 1024)
            a = rng.randint(0, npair, m)
            b = rng.randint(0, npair, m)
            keep = b <= a
            a, b = a[keep], b[keep]
            todo = np.unique(np.concatenate([a, b]))
            todo = todo[Q[todo] < 0]
            if len(todo):
                Q[todo] = pool.map(_q, pairs[todo], chunksize=64)
            ok = Q[a] * Q[b] >= 1e-12
            a, b = a[ok][:need], b[ok][:need]
            out.append(np.concatenate([pairs[a], pairs[b]], 1))
            need -= len(a)
            print('survivors', N - need, flush=True)
    qs = np.concatenate(out).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, 'c1_quartets.npz'), quartets=qs,
                        note=np.array('c1 seed 0, uniform unique quartets, Schwarz 1e-12 by libcint'))


if __name__ == '__main__':
    main()
