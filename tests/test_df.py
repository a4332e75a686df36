"""Density-fitted J (libcint_gb300/df.py) on the CPU: the packed-buffer index maps, rho weights,
metric mirroring and the two contractions, run on torch CPU tensors filled with the oracle's
int3c2e / int2c2e blocks in the plans' packed order, against dense einsums over the full
three-index tensor; and the fit against exact J from the oracle's ERIs through two properties that
hold for any auxiliary basis: Coulomb-metric fitting is variational (0 <= E_DF <= E_exact), and
exact when the density lies in the auxiliary span (an s x s product on one centre is the s
Gaussian of the summed exponent)."""
import numpy as np

from libcint_gb300 import df
from libcint_gb300 import molecules as M


def _system():
    mol, norb = M.config2(seed=1, natm=3, box=3.0)
    n = int(df._nsph(mol)[:norb].sum())
    d = np.random.RandomState(6).normal(0, 0.2, (n, n))
    return mol, norb, 0.5 * (d + d.T)


def _packed(oracle, name, mol, items):
    return np.concatenate([oracle.port.call(name, mol, tuple(int(x) for x in it))[1].ravel(order='F')
                           for it in items])


def _dense_df(oracle, mol, norb, dm):
    nsph = df._nsph(mol)
    loc = np.concatenate([[0], np.cumsum(nsph)])
    nao, naux = int(loc[norb]), int(loc[-1] - loc[norb])
    T3 = np.zeros((nao, nao, naux))
    for i in range(norb):
        for j in range(norb):
            for P in range(norb, mol.nbas):
                _, b = oracle.port.call('int3c2e_sph', mol, (i, j, P))
                T3[loc[i]:loc[i + 1], loc[j]:loc[j + 1], loc[P] - loc[norb]:loc[P + 1] - loc[norb]] = b
    V = np.zeros((naux, naux))
    for P in range(norb, mol.nbas):
        for Q in range(norb, mol.nbas):
            _, b = oracle.port.call('int2c2e_sph', mol, (P, Q))
            V[loc[P] - loc[norb]:loc[P + 1] - loc[norb], loc[Q] - loc[norb]:loc[Q + 1] - loc[norb]] = b
    rho = np.einsum('abp,ab->p', T3, dm)
    c = np.linalg.solve(V, rho)
    return T3, V, rho, np.einsum('abp,p->ab', T3, c)


def test_packed_df_matches_dense(oracle):
    import torch
    mol, norb, dm = _system()
    nsph = df._nsph(mol)
    loc = np.concatenate([[0], np.cumsum(nsph)])
    nao, naux = int(loc[norb]), int(loc[-1] - loc[norb])
    offs = loc[:-1].copy()
    offs[norb:] -= loc[norb]
    items3, items2 = df.df_items(norb, mol.nbas)
    T = torch.as_tensor(_packed(oracle, 'int3c2e_sph', mol, items3))
    v = torch.as_tensor(_packed(oracle, 'int2c2e_sph', mol, items2))
    pair_idx, aux_idx = df.packed_index(items3, nsph, offs, nao)
    vi, _ = df.packed_index(items2, nsph, offs, naux)
    assert len(pair_idx) == T.numel() and len(vi) == v.numel()
    w = torch.as_tensor(df.fit_weights(items3, nsph))
    V = df.mirror_metric(v, torch.as_tensor(vi), naux)
    _, Vref, rho_ref, Jref = _dense_df(oracle, mol, norb, dm)
    assert np.abs(V.numpy() - Vref).max() <= 1e-13 * np.abs(Vref).max()
    dmt = torch.as_tensor(dm)
    rho = df.contract_rho(T, w, torch.as_tensor(pair_idx), torch.as_tensor(aux_idx), dmt, naux)
    assert np.abs(rho.numpy() - rho_ref).max() <= 1e-13 * np.abs(rho_ref).max()
    c = torch.cholesky_solve(rho[:, None], torch.linalg.cholesky(V))[:, 0]
    diag = np.zeros((nao, nao), dtype=bool)
    for i in range(norb):
        diag[loc[i]:loc[i + 1], loc[i]:loc[i + 1]] = True
    J = df.contract_j(T, torch.as_tensor(pair_idx), torch.as_tensor(aux_idx), c, nao,
                      torch.as_tensor(diag)).numpy()
    assert np.abs(J - Jref).max() <= 1e-11 * np.abs(Jref).max()
    assert np.abs(J - J.T).max() <= 1e-14 * np.abs(Jref).max()


def _exact_j(oracle, mol, norb, dm):
    orb = M.Mol(mol.atm, mol.bas[:norb].copy(), mol.env, 'orbital')
    loc = orb.ao_loc()
    eri = np.zeros((loc[-1],) * 4)
    for q in M.unique_quartets(norb):
        i, j, k, l = (int(x) for x in q)
        _, blk = oracle.port.call('int2e_sph', orb, (i, j, k, l))
        for (a, b, c, d, t) in ((i, j, k, l, 'ijkl'), (j, i, k, l, 'jikl'), (i, j, l, k, 'ijlk'),
                                (j, i, l, k, 'jilk'), (k, l, i, j, 'klij'), (l, k, i, j, 'lkij'),
                                (k, l, j, i, 'klji'), (l, k, j, i, 'lkji')):
            eri[loc[a]:loc[a + 1], loc[b]:loc[b + 1], loc[c]:loc[c + 1], loc[d]:loc[d + 1]] = \
                np.transpose(blk, ['ijkl'.index(ch) for ch in t])
    return np.einsum('ijkl,kl->ij', eri, dm)


def test_df_is_variational(oracle):
    """E_DF = 1/2 rho V^-1 rho <= E_exact = 1/2 D J D for the same density (the fitted density's
    Coulomb error (rho - rho~|rho - rho~) >= 0), for a random positive semidefinite density"""
    mol, norb, _ = _system()
    n = int(df._nsph(mol)[:norb].sum())
    C = np.random.RandomState(8).normal(0, 0.3, (n, 4))
    dm = C @ C.T
    _, V, rho, Jdf = _dense_df(oracle, mol, norb, dm)
    Jx = _exact_j(oracle, mol, norb, dm)
    e_df = 0.5 * rho @ np.linalg.solve(V, rho)
    e_x = 0.5 * np.einsum('ij,ij', dm, Jx)
    assert np.isclose(e_df, 0.5 * np.einsum('ij,ij', dm, Jdf), rtol=1e-12)
    assert 0 < e_df <= e_x * (1 + 1e-12)


def test_df_exact_in_the_auxiliary_span(oracle):
    """Orbital s (exponent a) and p shells on two atoms; the auxiliary basis holds the s Gaussian
    of exponent 2a on the s shell's atom (plus p, d shells).  A density on the s x s element alone
    is fitted exactly, so DF J equals exact J for every orbital pair."""
    b = M._Builder()
    a0 = b.atom(1, (0.0, 0.0, 0.0))
    a1 = b.atom(1, (0.0, 0.4, 1.1))
    b.shell(a0, 0, [0.8], [M.gto_norm(0, 0.8)])
    b.shell(a1, 1, [0.6, 2.0], [M.gto_norm(1, 0.6) * 0.7, M.gto_norm(1, 2.0) * 0.4])
    b.shell(a1, 0, [1.3], [M.gto_norm(0, 1.3)])
    norb = 3
    b.shell(a0, 0, [1.6], [M.gto_norm(0, 1.6)])
    b.shell(a1, 1, [0.9], [M.gto_norm(1, 0.9)])
    b.shell(a0, 2, [1.1], [M.gto_norm(2, 1.1)])
    mol = b.mol('aux span')
    n = int(df._nsph(mol)[:norb].sum())
    dm = np.zeros((n, n))
    dm[0, 0] = 1.0
    _, _, _, Jdf = _dense_df(oracle, mol, norb, dm)
    Jx = _exact_j(oracle, mol, norb, dm)
    assert np.abs(Jdf - Jx).max() <= 1e-12 * np.abs(Jx).max()


def test_structured_index_equals_generic():
    """df_index (one slice per orbital pair) builds exactly packed_index's arrays for the
    df_items layout, for all pairs and for a subset"""
    mol, norb = M.config2(seed=2, natm=4, box=4.0)
    nsph = df._nsph(mol)
    loc = np.concatenate([[0], np.cumsum(nsph)])
    offs = loc[:-1].copy()
    offs[norb:] -= loc[norb]
    nao, naux = int(loc[norb]), int(loc[-1] - loc[norb])
    ii, jj = np.tril_indices(norb)
    full = np.stack([ii, jj], 1)
    for pairs in (full, full[::3]):
        items3, _ = df.df_items(norb, mol.nbas, pairs)
        a1, b1 = df.packed_index(items3, nsph, offs, nao)
        a2, b2 = df.df_index(pairs, nsph, offs, nao, naux)
        assert np.array_equal(a1, a2) and np.array_equal(b1, b2)


def _k_pieces(oracle, mol, norb):
    import torch
    nsph = df._nsph(mol)
    loc = np.concatenate([[0], np.cumsum(nsph)])
    offs = loc[:-1].copy()
    offs[norb:] -= loc[norb]
    nao, naux = int(loc[norb]), int(loc[-1] - loc[norb])
    ii, jj = np.tril_indices(norb)
    pairs = np.stack([ii, jj], 1)
    items3, items2 = df.df_items(norb, mol.nbas, pairs)
    T = torch.as_tensor(_packed(oracle, 'int3c2e_sph', mol, items3))
    pair_idx, aux_idx = df.df_index(pairs, nsph, offs, nao, naux)
    vi, _ = df.packed_index(items2, nsph, offs, naux)
    V = df.mirror_metric(torch.as_tensor(_packed(oracle, 'int2c2e_sph', mol, items2)),
                         torch.as_tensor(vi), naux)
    Bt = df.dense_fitted(T, torch.as_tensor(pair_idx), torch.as_tensor(aux_idx),
                         torch.linalg.cholesky(V), nao, naux)
    return Bt, nao


def test_df_k_matches_dense(oracle):
    """density-fitted K from the module's whitened tensor against the dense formula
    K = T V^-1 T contracted with D, on the oracle's blocks"""
    import torch
    mol, norb, dm = _system()
    Bt, _ = _k_pieces(oracle, mol, norb)
    T3, V, _, _ = _dense_df(oracle, mol, norb, dm)
    W = np.einsum('ijp,pq->ijq', T3, np.linalg.inv(V), optimize=True)
    Kref = np.einsum('ijq,jl,klq->ik', W, dm, T3, optimize=True)
    K = df.contract_k(Bt, torch.as_tensor(dm)).numpy()
    assert np.abs(K - Kref).max() <= 1e-10 * np.abs(Kref).max()
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(Kref).max()
    # the same tensor reproduces the fitted J
    _, _, _, Jref = _dense_df(oracle, mol, norb, dm)
    J = torch.einsum('qab,qcd,cd->ab', Bt, Bt, torch.as_tensor(dm)).numpy()
    assert np.abs(J - Jref).max() <= 1e-10 * np.abs(Jref).max()


def test_df_k_exact_in_the_auxiliary_span(oracle):
    """one orbital s shell (exponent a) and the auxiliary s Gaussian of exponent 2a on its atom:
    every orbital product is in the auxiliary span, so DF K equals exact K = (ss|ss) D"""
    import torch
    b = M._Builder()
    a0 = b.atom(1, (0.0, 0.0, 0.0))
    a1 = b.atom(1, (0.0, 0.4, 1.1))
    b.shell(a0, 0, [0.8], [M.gto_norm(0, 0.8)])
    b.shell(a0, 0, [1.6], [M.gto_norm(0, 1.6)])
    b.shell(a1, 1, [0.9], [M.gto_norm(1, 0.9)])
    mol = b.mol('aux span k')
    Bt, _ = _k_pieces(oracle, mol, 1)
    dm = np.array([[0.7]])
    K = df.contract_k(Bt, torch.as_tensor(dm)).numpy()
    _, eri = oracle.port.call('int2e_sph', M.Mol(mol.atm, mol.bas[:1].copy(), mol.env, 'o'),
                              (0, 0, 0, 0))
    assert abs(K[0, 0] - eri.ravel()[0] * 0.7) <= 1e-12 * abs(eri.ravel()[0])
