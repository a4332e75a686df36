"""Density fitting (RI) of the Coulomb and exchange matrices on the GPU, assembled from the
batched int3c2e and int2c2e plans:

    rho_Q = sum_cd (Q|cd) D_cd,   V c = rho  (V_PQ = (P|Q), Cholesky once per geometry),
    J_ab  = sum_P (ab|P) c_P.

The orbital and auxiliary shells live in one basis, as libcint's callers pass them to int3c2e_sph
/ int2c2e_sph (auxiliary shells after the orbital ones, src/cint3c2e.c:693-717,
src/cint2c2e.c:351-358).  The three-centre integrals of every orbital shell pair i >= j with every
auxiliary shell are computed once (the library's pipelined batch entry: chunk plans built on host
threads while the GPU runs earlier chunks) and stay in HBM in the plans' packed layout (blocks (di, dj, dP) back to
back, i fastest: pair p owns di dj naux doubles).  A J build is two passes of the library's DF
kernels over that buffer (cintgpu_df_rho, cintgpu_df_j: per-pair descriptors only, no per-element
index arrays, no atomics on J) around a triangular solve.  K uses the buffer scattered into a
dense (naux, nao, nao) tensor whitened by the metric's Cholesky factor: K = sum_q B~_q D B~_q^T
(small systems).  Densities, J and K are spherical (libcint's int2e_sph AO order).

The per-element formulation (packed_index, fit_weights, contract_rho, contract_j: gathers and
scatter-adds in torch) states the same contractions densely; the CPU tests check it against
einsums over the oracle's full tensor and the GPU tests check the kernels against it.
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
    pairs: orbital shell pairs (i >= j) to include (default: all).  chunk: (ij|P) triples per
    call of the batch entry while the buffer is built."""

    def __init__(self, mol, norb, pairs=None, chunk=40_000_000):
        import ctypes

        import torch
        from . import INT2C2E_SPH, INT3C2E_SPH, Plan, _check, _ptr, batch_device, lib
        self.mol, self.norb = mol, norb
        nsph = _nsph(mol)
        loc = np.concatenate([[0], np.cumsum(nsph)])
        self.nao = int(loc[norb])
        self.naux = int(loc[-1] - loc[norb])
        offs = loc[:-1].copy()
        offs[norb:] -= loc[norb]                          # auxiliary functions counted from 0
        self._nsph, self._offs = nsph, offs
        if pairs is None:
            ii, jj = np.tril_indices(norb)
            pairs = np.stack([ii, jj], 1)
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        if len(pairs) and (pairs.min() < 0 or pairs.max() >= norb):
            raise ValueError('pairs must index orbital shells 0..norb-1')
        self.pairs = pairs
        desc = np.ascontiguousarray(np.stack([offs[pairs[:, 0]], offs[pairs[:, 1]], nsph[pairs[:, 0]],
                                              nsph[pairs[:, 1]]], 1), dtype=np.int32)
        L = lib()
        h = ctypes.c_void_p()
        _check(L.cintgpu_df_create(ctypes.byref(h), _ptr(desc), len(pairs), self.nao, self.naux),
               'cintgpu_df_create')
        self._df = h
        size = int(L.cintgpu_df_size(h))
        self.T = torch.empty(max(size, 1), dtype=torch.float64, device='cuda')
        # (ij|P) through the library's pipelined batch entry (chunk plans built on host threads
        # while the GPU runs earlier chunks, reused device slots), in calls of whole pairs so the
        # item list on the host stays bounded
        seg = nsph[pairs[:, 0]] * nsph[pairs[:, 1]] * self.naux
        start = np.concatenate([[0], np.cumsum(seg)])
        naux_sh = mol.nbas - norb
        per = max(1, chunk // max(naux_sh, 1))
        for a in range(0, len(pairs), per):
            b = min(a + per, len(pairs))
            items3, _ = df_items(norb, mol.nbas, pairs[a:b])
            batch_device(INT3C2E_SPH, mol, items3, self.T.narrow(0, int(start[a]), int(start[b] - start[a])))
        # the metric over auxiliary pairs P >= Q, mirrored into a dense matrix
        _, items2 = df_items(norb, mol.nbas, pairs[:0])
        p2 = Plan(INT2C2E_SPH, mol, items2)
        v = torch.empty(p2.output_size, dtype=torch.float64, device='cuda')
        p2.execute(v)
        torch.cuda.synchronize()
        p2.close()
        vi, _ = packed_index(items2, nsph, offs, self.naux)
        if len(vi) != v.numel() or (len(vi) and vi.max() >= self.naux * self.naux):
            raise ValueError('metric index map does not match the (P|Q) buffer')
        self.V = mirror_metric(v, torch.as_tensor(vi, device=v.device), self.naux)
        self.L = torch.linalg.cholesky(self.V)

    def _dev(self, x, shape, name):
        import torch
        if not (torch.is_tensor(x) and x.is_cuda and x.dtype == torch.float64 and tuple(x.shape) == shape):
            raise ValueError('%s must be a CUDA float64 tensor of shape %s' % (name, shape))
        return x.contiguous()

    def rho(self, dm):
        """rho_Q = sum_cd (Q|cd) D_cd for the symmetric spherical density dm (CUDA tensor)."""
        import ctypes

        import torch
        from . import _check, lib
        dm = self._dev(dm, (self.nao, self.nao), 'dm')
        r = torch.empty(self.naux, dtype=torch.float64, device=dm.device)
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _check(lib().cintgpu_df_rho(self._df, ctypes.c_void_p(self.T.data_ptr()),
                                    ctypes.c_void_p(dm.data_ptr()), ctypes.c_void_p(r.data_ptr()), st),
               'cintgpu_df_rho')
        return r

    def coefficients(self, dm):
        import torch
        r = self.rho(dm)
        return torch.cholesky_solve(r[:, None], self.L)[:, 0]

    def vj(self, dm):
        """Density-fitted J (spherical) for the symmetric density dm (CUDA tensor)."""
        return self.vj_from_coefficients(self.coefficients(dm))

    def vj_from_coefficients(self, c):
        """J_ab = sum_P (ab|P) c_P for fitting coefficients c (CUDA tensor of naux)."""
        import ctypes

        import torch
        from . import _check, lib
        c = self._dev(c, (self.naux,), 'c')
        J = torch.empty(self.nao, self.nao, dtype=torch.float64, device=c.device)
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _check(lib().cintgpu_df_j(self._df, ctypes.c_void_p(self.T.data_ptr()), ctypes.c_void_p(c.data_ptr()),
                                  ctypes.c_void_p(J.data_ptr()), st), 'cintgpu_df_j')
        return J

    def index_maps(self):
        """(pair_idx, aux_idx) device tensors of the packed buffer (per-element AO pair and
        auxiliary function, df_index), built on first use: K and the dense formulation need
        them, J does not."""
        import torch
        if getattr(self, '_maps', None) is None:
            pi, ai = df_index(self.pairs, self._nsph, self._offs, self.nao, self.naux)
            self._maps = (torch.as_tensor(pi, device=self.T.device), torch.as_tensor(ai, device=self.T.device))
        return self._maps

    def vk(self, dm):
        """Density-fitted K (spherical) for the symmetric density dm; the whitened three-index
        tensor (naux * nao^2 doubles) is formed on first use and kept."""
        if getattr(self, 'Bt', None) is None:
            pair_idx, aux_idx = self.index_maps()
            self.Bt = dense_fitted(self.T, pair_idx, aux_idx, self.L, self.nao, self.naux)
        return contract_k(self.Bt, dm)

    def close(self):
        if getattr(self, '_df', None):
            from . import lib
            lib().cintgpu_df_destroy(self._df)
            self._df = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
