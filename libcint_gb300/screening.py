"""Integral screening for the J/K contractions (the direct-SCF loop of a libcint caller).

Cauchy-Schwarz: |(ab|cd)| <= sqrt((ab|ab)) sqrt((cd|cd)), so each shell pair gets
Q_ij = max over a in i, b in j of sqrt(|(ab|ab)|), from the diagonal elements of the (ij|ij)
blocks (one int2e_sph plan over the diagonal quartets).  A unique quartet (ij|kl) then contributes
at most Q_ij Q_kl times a density element to J (D_kl to J_ij, D_ij to J_kl) and to K (D_jl, D_jk,
D_il, D_ik); it is dropped when that bound, with the largest density element of the blocks it
touches, is below the threshold.  Densities are spherical (libcint's int2e_sph AO order).
"""
import numpy as np

from .molecules import shell_nsph as _nsph


def diagonal_pairs(nbas):
    """Shell pairs i >= j and their diagonal quartets (i, j, i, j)."""
    ii, jj = np.tril_indices(nbas)
    pairs = np.stack([ii, jj], 1)
    return pairs, np.concatenate([pairs, pairs], 1).astype(np.int32)


def diagonal_index(mol, pairs):
    """Positions of the (ab|ab) elements inside the packed (ij|ij) blocks (blocks back to back,
    Fortran order (di, dj, di, dj)), and each pair's count of them (di dj)."""
    n = _nsph(mol)
    di, dj = n[pairs[:, 0]], n[pairs[:, 1]]
    size = (di * dj) ** 2
    start = np.concatenate([[0], np.cumsum(size)[:-1]])
    cnt = di * dj
    blk = np.repeat(np.arange(len(pairs)), cnt)
    t = np.arange(int(cnt.sum())) - np.repeat(np.concatenate([[0], np.cumsum(cnt)[:-1]]), cnt)
    a, b = t % di[blk], t // di[blk]
    d0, d1 = di[blk], dj[blk]
    pos = start[blk] + a + d0 * (b + d1 * (a + d0 * b))
    return pos, cnt


def schwarz_from_diagonal(nbas, pairs, diag, cnt):
    """Q (nbas x nbas, symmetric) from the (ab|ab) elements grouped per pair."""
    seg = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    m = np.maximum.reduceat(np.sqrt(np.abs(diag)), seg) if len(diag) else np.zeros(0)
    Q = np.zeros((nbas, nbas))
    Q[pairs[:, 0], pairs[:, 1]] = m
    Q[pairs[:, 1], pairs[:, 0]] = m
    return Q


def pair_bounds(mol, pairs):
    """Q for the given shell pairs (rows (i, j)): sqrt(max |(ab|ab)|) over the pair's functions,
    from one int2e_sph plan over the diagonal quartets (i, j, i, j) on the GPU."""
    import torch
    from . import INT2E_SPH, Plan
    pairs = np.ascontiguousarray(pairs, dtype=np.int64).reshape(-1, 2)
    items = np.concatenate([pairs, pairs], 1).astype(np.int32)
    plan = Plan(INT2E_SPH, mol, items)
    out = torch.empty(plan.output_size, dtype=torch.float64, device='cuda')
    plan.execute(out)
    pos, cnt = diagonal_index(mol, pairs)
    if len(pos) and (pos.min() < 0 or pos.max() >= plan.output_size):   # checked on the host
        raise ValueError('diagonal positions outside the plan output')
    diag = out[torch.as_tensor(pos, device=out.device)].cpu().numpy()
    plan.close()
    seg = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    return np.maximum.reduceat(np.sqrt(np.abs(diag)), seg) if len(diag) else np.zeros(0)


def schwarz_bounds(mol):
    """Q_ij for every shell pair (nbas x nbas, symmetric), from one int2e_sph plan over the
    diagonal quartets (GPU)."""
    pairs, _ = diagonal_pairs(mol.nbas)
    m = pair_bounds(mol, pairs)
    Q = np.zeros((mol.nbas, mol.nbas))
    Q[pairs[:, 0], pairs[:, 1]] = m
    Q[pairs[:, 1], pairs[:, 0]] = m
    return Q


def shell_density_max(mol, dm):
    """max |D| over each shell-pair block of a spherical density (numpy or torch)."""
    d = dm.detach().abs().cpu().numpy() if hasattr(dm, 'detach') else np.abs(np.asarray(dm))
    loc = np.concatenate([[0], np.cumsum(_nsph(mol))])
    rows = np.maximum.reduceat(d, loc[:-1], axis=0)
    return np.maximum.reduceat(rows, loc[:-1], axis=1)


def screen_quartets(quartets, Q, Dmax, threshold, with_j=True, with_k=True):
    """The unique quartets whose Schwarz bound times the density they meet reaches threshold."""
    q = np.asarray(quartets, dtype=np.int64).reshape(-1, 4)
    i, j, k, l = q.T
    bound = Q[i, j] * Q[k, l]
    dens = np.zeros(len(q))
    if with_j:
        dens = np.maximum(dens, np.maximum(Dmax[k, l], Dmax[i, j]))
    if with_k:
        dens = np.maximum.reduce([dens, Dmax[j, l], Dmax[j, k], Dmax[i, l], Dmax[i, k]])
    return q[bound * dens >= threshold]


def screened_coulomb_plans(mol, dm, threshold, Q=None, with_j=True, with_k=True):
    """CoulombPlans over the unique quartets that survive screening for the density dm (Q from
    schwarz_bounds when not given; keep it across densities of one geometry)."""
    from .coulomb import CoulombPlans
    from .molecules import unique_quartets
    Q = schwarz_bounds(mol) if Q is None else Q
    qs = screen_quartets(unique_quartets(mol.nbas), Q, shell_density_max(mol, dm), threshold,
                         with_j, with_k)
    return CoulombPlans(mol, qs)
