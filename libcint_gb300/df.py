"""Density fitting (RI) of the Coulomb and exchange matrices on the GPU, assembled from the
batched int3c2e and int2c2e plans:

    rho_Q = sum_cd (Q|cd) D_cd,   V c = rho  (V_PQ = (P|Q), Cholesky once per geometry),
    J_ab  = sum_P (ab|P) c_P.

The orbital and auxiliary shells live in one basis, as libcint's callers pass them to int3c2e_sph
/ int2c2e_sph (auxiliary shells after the orbital ones, src/cint3c2e.c:693-717,
src/cint2c2e.c:351-358).  The three-centre integrals of every orbital shell pair i >= j with every
auxiliary shell are computed once by one plan and stay in HBM in the plan's packed layout (blocks
(di, dj, dP) back to back, i fastest); host-built index maps give each packed element its AO pair
and auxiliary function, so a J build is two gathers and two scatter-adds over that buffer plus a
triangular solve.  K uses the buffer scattered into a dense (naux, nao, nao) tensor whitened by
the metric's Cholesky factor: K = sum_q B~_q D B~_q^T.  Densities, J and K are spherical
(libcint's int2e_sph AO order).
"""
import numpy as np

from .molecules import shell_nsph as _nsph


def packed_index(items, dims, offs, nao):
    """For blocks laid out back to back (item q: extents dims[items[q, k]] per shell k, first index
    fastest), the flat (row-major, leading dimension nao) AO index of shells 0 and 1 and the index
    along shell 2 of every element.  items: (n, 2) or (n, 3) shell indices; dims, offs: per shell
    extent and first function index.  Returns (pair_index, third_index or None), int64."""
    items = np.asarray(items, dtype=np.int64)
    d = dims[items]                                   # (n, k) extents per block
    sizes = np.prod(d, axis=1)
    start = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    blk = np.repeat(np.arange(len(items)), sizes)
    t = np.arange(int(sizes.sum()), dtype=np.int64) - start[blk]
    d0, d1 = d[blk, 0], d[blk, 1]
    a = t % d0
    b = (t // d0) % d1
    pair = (offs[items[blk, 0]] + a) * nao + offs[items[blk, 1]] + b
    if items.shape[1] == 2:
        return pair, None
    return pair, offs[items[blk, 2]] + t // (d0 * d1)


def df_items(norb, nbas, pairs=None):
    """(items3, items2): the (i, j, P) triples of every listed orbital pair i >= j (default: all)
    with every auxiliary shell P (pair-major), and the auxiliary pairs P >= Q of the metric."""
    aux = np.arange(norb, nbas, dtype=np.int64)
    if pairs is None:
        ii, jj = np.tril_indices(norb)
        pairs = np.stack([ii, jj], 1)
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    items3 = np.concatenate([np.repeat(pairs, len(aux), axis=0),
                             np.tile(aux, len(pairs))[:, None]], 1).astype(np.int32)
    pi, qi = np.tril_indices(len(aux))
    items2 = np.stack([aux[pi], aux[qi]], 1).astype(np.int32)
    return items3, items2


def df_index(pairs, nsph, offs, nao, naux):
    """packed_index for the df_items layout, by its structure: orbital pair p's (ij|P) blocks over
    all auxiliary shells form one segment of naux * di * dj elements in which the di * dj AO-pair
    pattern (i fastest) repeats for every auxiliary function.  Same arrays, built by one slice
    assignment per pair instead of per-element arithmetic."""
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    di, dj = nsph[pairs[:, 0]], nsph[pairs[:, 1]]
    seg = di * dj * naux
    start = np.concatenate([[0], np.cumsum(seg)])
    pair = np.empty(int(start[-1]), dtype=np.int64)
    aux = np.empty(int(start[-1]), dtype=np.int64)
    aux_pattern = {}
    for p, (i, j) in enumerate(pairs):
        a, b = int(di[p]), int(dj[p])
        ab = (offs[i] + np.arange(a))[:, None] * nao + (offs[j] + np.arange(b))[None, :]
        s0, s1 = int(start[p]), int(start[p + 1])
        pair[s0:s1] = np.tile(ab.ravel(order='F'), naux)
        if a * b not in aux_pattern:
            aux_pattern[a * b] = np.repeat(np.arange(naux, dtype=np.int64), a * b)
        aux[s0:s1] = aux_pattern[a * b]
    return pair, aux


def fit_weights(items3, nsph):
    """Per packed element of the (ij|P) buffer: 2 for a pair of two different shells (it stands
    for (ab|P) and (ba|P) in rho), else 1."""
    items3 = np.asarray(items3, dtype=np.int64)
    blk_w = np.where(items3[:, 0] != items3[:, 1], 2.0, 1.0)
    return np.repeat(blk_w, np.prod(nsph[items3], axis=1))


def mirror_metric(v, vi, naux):
    """Dense symmetric metric from the packed P >= Q blocks v at flat indices vi (torch)."""
    import torch
    V = torch.zeros(naux * naux, dtype=v.dtype, device=v.device)
    filled = torch.zeros(naux * naux, dtype=torch.bool, device=v.device)
    V[vi] = v
    filled[vi] = True
    V, filled = V.view(naux, naux), filled.view(naux, naux)
    return torch.where(filled, V, V.T)


def contract_rho(T, w, pair_idx, aux_idx, dm, naux):
    """rho_Q = sum_cd (Q|cd) D_cd from the packed (ij|P) buffer (torch, any device)."""
    import torch
    vals = T * w * dm.reshape(-1)[pair_idx]
    return torch.zeros(naux, dtype=T.dtype, device=T.device).index_add_(0, aux_idx, vals)


def contract_j(T, pair_idx, aux_idx, c, nao, diag):
    """J_ab = sum_P (ab|P) c_P for the listed pairs (i >= j), symmetrised: X + X^T minus the
    diagonal shell blocks (held whole in X)."""
    import torch
    X = torch.zeros(nao * nao, dtype=T.dtype, device=T.device).index_add_(
        0, pair_idx, T * c[aux_idx]).view(nao, nao)
    return X + X.T - torch.where(diag, X, torch.zeros_like(X))


def dense_fitted(T, pair_idx, aux_idx, L, nao, naux):
    """B~ = L^-1 B with B[q, a, b] = (ab|q) for every AO pair (both orders) from the packed (ij|P)
    buffer, L the metric's Cholesky factor: (naux, nao, nao), so that (ab|cd) ~ sum_q
    B~[q, a, b] B~[q, c, d].  Memory naux * nao^2 doubles (torch, any device)."""
    import torch
    B = torch.zeros(naux * nao * nao, dtype=T.dtype, device=T.device)
    a, b = pair_idx // nao, pair_idx % nao
    B[aux_idx * (nao * nao) + pair_idx] = T
    B[aux_idx * (nao * nao) + b * nao + a] = T          # the (ba|q) half (same values)
    B = torch.linalg.solve_triangular(L, B.view(naux, nao * nao), upper=False)
    return B.view(naux, nao, nao)


def contract_k(Bt, dm):
    """K[i, k] = sum_q sum_jl B~[q, i, j] D[j, l] B~[q, k, l] (density-fitted exchange)."""
    naux, nao, _ = Bt.shape
    X = (Bt.reshape(naux * nao, nao) @ dm).view(naux, nao, nao)          # X_q = B~_q D
    return X.permute(1, 0, 2).reshape(nao, naux * nao) @ Bt.permute(1, 0, 2).reshape(nao, naux * nao).T


class DFCoulomb:
    """RI-J for one geometry: orbital shells 0..norb-1, auxiliary shells norb..nbas-1 of mol.
    pairs: orbital shell pairs (i >= j) to include (default: all)."""

    def __init__(self, mol, norb, pairs=None):
        import torch
        from . import INT2C2E_SPH, INT3C2E_SPH, Plan
        self.mol, self.norb = mol, norb
        nsph = _nsph(mol)
        loc = np.concatenate([[0], np.cumsum(nsph)])
        self.nao = int(loc[norb])
        self.naux = int(loc[-1] - loc[norb])
        offs = loc[:-1].copy()
        offs[norb:] -= loc[norb]                          # auxiliary functions counted from 0
        if pairs is None:
            ii, jj = np.tril_indices(norb)
            pairs = np.stack([ii, jj], 1)
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        items3, items2 = df_items(norb, mol.nbas, pairs)
        p3 = Plan(INT3C2E_SPH, mol, items3)
        self.T = torch.empty(p3.output_size, dtype=torch.float64, device='cuda')
        p3.execute(self.T)
        pair_idx, aux_idx = df_index(pairs, nsph, offs, self.nao, self.naux)
        if len(pair_idx) != self.T.numel() or (len(pair_idx) and (
                pair_idx.max() >= self.nao * self.nao or aux_idx.max() >= self.naux)):
            raise ValueError('index maps do not match the (ij|P) buffer')   # host-side check
        dev = self.T.device
        self.pair_idx = torch.as_tensor(pair_idx, device=dev)
        self.aux_idx = torch.as_tensor(aux_idx, device=dev)
        self.w = torch.as_tensor(fit_weights(items3, nsph), device=dev)
        # the metric over auxiliary pairs P >= Q, mirrored into a dense matrix
        p2 = Plan(INT2C2E_SPH, mol, items2)
        v = torch.empty(p2.output_size, dtype=torch.float64, device='cuda')
        p2.execute(v)
        torch.cuda.synchronize()                          # both plans done before they are freed
        p3.close()
        p2.close()
        vi, _ = packed_index(items2, nsph, offs, self.naux)
        if len(vi) != v.numel() or (len(vi) and vi.max() >= self.naux * self.naux):
            raise ValueError('metric index map does not match the (P|Q) buffer')
        self.V = mirror_metric(v, torch.as_tensor(vi, device=dev), self.naux)
        self.L = torch.linalg.cholesky(self.V)
        diag = np.zeros((self.nao, self.nao), dtype=bool)
        for i in range(norb):
            diag[loc[i]:loc[i + 1], loc[i]:loc[i + 1]] = True
        self.diag = torch.as_tensor(diag, device=dev)

    def rho(self, dm):
        """rho_Q = sum_cd (Q|cd) D_cd for the symmetric spherical density dm (torch, cuda)."""
        return contract_rho(self.T, self.w, self.pair_idx, self.aux_idx, dm, self.naux)

    def coefficients(self, dm):
        import torch
        r = self.rho(dm)
        return torch.cholesky_solve(r[:, None], self.L)[:, 0]

    def vj(self, dm):
        """Density-fitted J (spherical) for the symmetric density dm."""
        return contract_j(self.T, self.pair_idx, self.aux_idx, self.coefficients(dm), self.nao,
                          self.diag)

    def vk(self, dm):
        """Density-fitted K (spherical) for the symmetric density dm; the whitened three-index
        tensor (naux * nao^2 doubles) is formed on first use and kept."""
        if getattr(self, 'Bt', None) is None:
            self.Bt = dense_fitted(self.T, self.pair_idx, self.aux_idx, self.L, self.nao, self.naux)
        return contract_k(self.Bt, dm)
