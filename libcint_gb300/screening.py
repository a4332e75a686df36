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


def pair_bounds(mol, pairs, chunk=250000):
    """Q for the given shell pairs (rows (i, j)): sqrt(max |(ab|ab)|) over the pair's functions,
    from int2e_sph plans over the diagonal quartets (i, j, i, j) on the GPU, `chunk` pairs per
    plan (so millions of pairs do not need one plan's host and device tables at once)."""
    pairs = np.ascontiguousarray(pairs, dtype=np.int64).reshape(-1, 2)
    if len(pairs) > chunk:
        return np.concatenate([pair_bounds(mol, pairs[a:a + chunk], chunk)
                               for a in range(0, len(pairs), chunk)])
    import torch
    from . import INT2E_SPH, Plan
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


class ScreenedCoulomb:
    """Whole-molecule J / K / adjoint over the Schwarz-surviving unique quartets, never stored.

    The shell pairs i >= j with their bounds Q (pair_bounds, one GPU plan) are handed to
    cintgpu_screened_run, which orders them by Q, enumerates the quartets (P, Q) with
    Q_P Q_Q >= threshold bra row by bra row (binary search per row), builds chunk plans on host
    threads and accumulates the contraction on the GPU; no quartet list and no (ij|kl) is kept.
    bra_range = (p0, p1) restricts the bra pairs to positions [p0, p1) of the Q order (a slab, for
    timing a fixed fraction of a large molecule)."""

    def __init__(self, mol, threshold=1e-12, Q=None):
        import torch
        from .coulomb import cart2sph_matrix, _shell_diag_mask
        self.mol = mol
        self.threshold = float(threshold)
        ii, jj = np.tril_indices(mol.nbas)
        self.pairs = np.ascontiguousarray(np.stack([ii, jj], 1), dtype=np.int32)
        self.q = np.ascontiguousarray(pair_bounds(mol, self.pairs) if Q is None else Q[ii, jj],
                                      dtype=np.float64)
        self.C = torch.as_tensor(cart2sph_matrix(mol), device='cuda')
        self.diag = torch.as_tensor(_shell_diag_mask(mol, cart=True), device='cuda')
        self.last_quartets = 0

    def _run(self, kind, dmc, vj=None, vk=None, g=None, ga=None, bra_range=None):
        import ctypes
        from . import _check, _ptr, lib
        mol = self.mol
        p0, p1 = (0, len(self.pairs)) if bra_range is None else bra_range
        n = ctypes.c_int64(0)
        P = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
        L = lib()
        _check(L.cintgpu_screened_run(kind, _ptr(self.pairs), _ptr(self.q), len(self.pairs),
                                      ctypes.c_double(self.threshold), ctypes.c_int64(p0),
                                      ctypes.c_int64(p1), _ptr(mol.atm), mol.natm, _ptr(mol.bas),
                                      mol.nbas, _ptr(mol.env), P(dmc), P(vj), P(vk), P(g), P(ga),
                                      ctypes.byref(n)), 'cintgpu_screened_run')
        self.last_quartets = int(n.value)

    def dm_cart(self, dm):
        """the spherical density in the Cartesian AO basis the kernels contract with"""
        return (self.C.T @ dm @ self.C).contiguous()

    def get_jk(self, dm, with_j=True, with_k=True, bra_range=None):
        import torch
        from .coulomb import J_BUILD, JK_BUILD, K_BUILD
        kind = JK_BUILD if (with_j and with_k) else (J_BUILD if with_j else K_BUILD)
        dmc = self.dm_cart(dm)
        XJ = torch.zeros_like(dmc) if with_j else None
        XK = torch.zeros_like(dmc) if with_k else None
        self._run(kind, dmc, XJ, XK, bra_range=bra_range)
        J = K = None
        if with_j:
            J = self.C @ (XJ + XJ.T - torch.where(self.diag, XJ, torch.zeros_like(XJ))) @ self.C.T
        if with_k:
            K = self.C @ (XK + XK.T) @ self.C.T
        return J, K

    def grad(self, dm, with_exponents=False, bra_range=None):
        """(dL/dR (natm, 3), dL/dalpha or None) for L = 1/2 D (ij|kl) D over the screened list."""
        import torch
        from .coulomb import J_GRAD, J_GRAD_EXP
        from .molecules import NPRIM_OF
        dmc = self.dm_cart(dm)
        g = torch.zeros((self.mol.natm, 3), dtype=torch.float64, device='cuda')
        ga = (torch.zeros(int(self.mol.bas[:, NPRIM_OF].sum()), dtype=torch.float64, device='cuda')
              if with_exponents else None)
        self._run(J_GRAD_EXP if with_exponents else J_GRAD, dmc, g=g, ga=ga, bra_range=bra_range)
        return g, ga


def screened_list(Q_pairs, pairs, threshold):
    """The quartets ScreenedCoulomb evaluates, materialised (for tests on small systems): pairs
    ordered by Q (largest first, stable), then (p, q) with q <= p and Q_p Q_q >= threshold."""
    order = np.argsort(-np.asarray(Q_pairs), kind='stable')
    qs = np.asarray(Q_pairs)[order]
    out = []
    for p in range(len(order)):
        k = np.nonzero(qs[:p + 1] * qs[p] >= threshold)[0]
        for t in k:
            out.append(np.concatenate([pairs[order[p]], pairs[order[t]]]))
    return np.array(out, dtype=np.int32).reshape(-1, 4)
