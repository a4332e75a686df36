"""Schwarz / density screening of the J/K contractions (libcint_gb300/screening.py) on the CPU,
with the oracle's blocks standing in for the GPU plan's output: the (ab|ab) extraction from packed
(ij|ij) blocks, the Cauchy-Schwarz bound on every unique quartet, and the error of J and K over a
screened list against the full list, bounded by the dropped quartets' bounds."""
import numpy as np

from libcint_gb300 import molecules as M
from libcint_gb300 import screening as S
from tests.test_jk_algebra import _contract


def _mol():
    return M.config3(seed=5, natm=4, box=9.0)


def _blocks(oracle, mol):
    return {tuple(int(x) for x in q): oracle.port.call('int2e_sph', mol, q)[1]
            for q in M.unique_quartets(mol.nbas)}


def test_schwarz_from_packed_diagonal(oracle):
    mol = _mol()
    pairs, items = S.diagonal_pairs(mol.nbas)
    packed = np.concatenate([oracle.port.call('int2e_sph', mol, it)[1].ravel(order='F') for it in items])
    pos, cnt = S.diagonal_index(mol, pairs)
    Q = S.schwarz_from_diagonal(mol.nbas, pairs, packed[pos], cnt)
    for i, j in pairs:
        _, b = oracle.port.call('int2e_sph', mol, (i, j, i, j))
        want = np.sqrt(np.abs(np.einsum('abab->ab', b)).max())
        assert Q[i, j] == Q[j, i] == want


def test_schwarz_bounds_every_quartet(oracle):
    mol = _mol()
    pairs, items = S.diagonal_pairs(mol.nbas)
    packed = np.concatenate([oracle.port.call('int2e_sph', mol, it)[1].ravel(order='F') for it in items])
    pos, cnt = S.diagonal_index(mol, pairs)
    Q = S.schwarz_from_diagonal(mol.nbas, pairs, packed[pos], cnt)
    for (i, j, k, l), blk in _blocks(oracle, mol).items():
        assert np.abs(blk).max() <= Q[i, j] * Q[k, l] * (1 + 1e-12)


def test_screened_jk_error_is_bounded(oracle):
    mol = _mol()
    blocks = _blocks(oracle, mol)
    pairs, _ = S.diagonal_pairs(mol.nbas)
    Q = np.zeros((mol.nbas, mol.nbas))
    for i, j in pairs:
        Q[i, j] = Q[j, i] = np.sqrt(np.abs(np.einsum('abab->ab', blocks[(i, j, i, j)])).max())
    n = mol.ao_loc()[-1]
    d = np.random.RandomState(3).normal(0, 0.2, (n, n))
    dm = 0.5 * (d + d.T)
    Dmax = S.shell_density_max(mol, dm)
    qs = M.unique_quartets(mol.nbas)
    assert len(S.screen_quartets(qs, Q, Dmax, 0.0)) == len(qs)
    J0, K0 = _contract(mol, blocks, dm, kernel_order=False)
    nmax = max(b.size for b in blocks.values())
    dropped_any = False
    for thr in (1e-12, 1e-9, 1e-6):
        kept = S.screen_quartets(qs, Q, Dmax, thr)
        kept_set = {tuple(int(x) for x in q) for q in kept}
        drop = [q for q in blocks if q not in kept_set]
        dropped_any |= len(drop) > 0
        J, K = _contract(mol, {q: blocks[q] for q in kept_set}, dm, kernel_order=False)
        # each dropped quartet moves an element of J or K by at most 8 bound x density x block size
        budget = sum(8 * Q[i, j] * Q[k, l] * Dmax.max() * nmax for (i, j, k, l) in drop)
        per_q = [Q[i, j] * Q[k, l] * max(Dmax[k, l], Dmax[i, j], Dmax[j, l], Dmax[j, k], Dmax[i, l],
                                         Dmax[i, k]) for (i, j, k, l) in drop]
        assert all(p < thr for p in per_q)
        assert np.abs(J - J0).max() <= budget + 1e-15 and np.abs(K - K0).max() <= budget + 1e-15
    assert dropped_any
