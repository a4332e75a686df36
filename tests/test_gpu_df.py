"""Density-fitted J on the GPU (libcint_gb300/df.py: int3c2e and int2c2e plans, packed-buffer
contractions, Cholesky of the metric) against the same fit from the oracle's blocks in dense
numpy, and exact where the density lies in the auxiliary span.  Tolerance 1e-10 of max |J|: the
fit moves 1e-14 rounding of V or (ij|P) by ~3e-13 of J on these bases (metric condition ~3e4)."""
import numpy as np
import pytest

from libcint_gb300 import df
from libcint_gb300 import molecules as M
from tests.test_df import _dense_df, _exact_j

pytestmark = pytest.mark.gpu


def test_df_j_matches_oracle_fit(gpulib, oracle):
    import torch
    mol, norb = M.config2(seed=1, natm=2, box=3.0)
    n = int(df._nsph(mol)[:norb].sum())
    d = np.random.RandomState(6).normal(0, 0.2, (n, n))
    dm = 0.5 * (d + d.T)
    fit = df.DFCoulomb(mol, norb)
    J = fit.vj(torch.as_tensor(dm, device='cuda')).cpu().numpy()
    _, V, rho, Jref = _dense_df(oracle, mol, norb, dm)
    assert np.abs(fit.V.cpu().numpy() - V).max() <= 1e-12 * np.abs(V).max()
    assert np.abs(fit.rho(torch.as_tensor(dm, device='cuda')).cpu().numpy() - rho).max() \
        <= 1e-12 * np.abs(rho).max()
    assert np.abs(J - Jref).max() <= 1e-10 * np.abs(Jref).max()


def test_df_j_exact_in_span_gpu(gpulib, oracle):
    import torch
    b = M._Builder()
    a0 = b.atom(1, (0.0, 0.0, 0.0))
    a1 = b.atom(1, (0.0, 0.4, 1.1))
    b.shell(a0, 0, [0.8], [M.gto_norm(0, 0.8)])
    b.shell(a1, 1, [0.6, 2.0], [M.gto_norm(1, 0.6) * 0.7, M.gto_norm(1, 2.0) * 0.4])
    b.shell(a1, 0, [1.3], [M.gto_norm(0, 1.3)])
    b.shell(a0, 0, [1.6], [M.gto_norm(0, 1.6)])
    b.shell(a1, 1, [0.9], [M.gto_norm(1, 0.9)])
    b.shell(a0, 2, [1.1], [M.gto_norm(2, 1.1)])
    mol = b.mol('aux span')
    norb = 3
    n = int(df._nsph(mol)[:norb].sum())
    dm = np.zeros((n, n))
    dm[0, 0] = 1.0
    J = df.DFCoulomb(mol, norb).vj(torch.as_tensor(dm, device='cuda')).cpu().numpy()
    Jx = _exact_j(oracle, mol, norb, dm)
    assert np.abs(J - Jx).max() <= 1e-12 * np.abs(Jx).max()


def test_df_k_matches_oracle_fit(gpulib, oracle):
    """density-fitted K on the GPU (whitened three-index tensor formed from the int3c2e plan's
    packed buffer, then two batched products) against K = T V^-1 T contracted with D on the
    oracle's blocks in dense numpy; K symmetric"""
    import torch
    mol, norb = M.config2(seed=1, natm=2, box=3.0)
    n = int(df._nsph(mol)[:norb].sum())
    d = np.random.RandomState(7).normal(0, 0.2, (n, n))
    dm = 0.5 * (d + d.T)
    fit = df.DFCoulomb(mol, norb)
    K = fit.vk(torch.as_tensor(dm, device='cuda')).cpu().numpy()
    T3, V, _, _ = _dense_df(oracle, mol, norb, dm)
    W = np.einsum('ijp,pq->ijq', T3, np.linalg.inv(V), optimize=True)
    Kref = np.einsum('ijq,jl,klq->ik', W, dm, T3, optimize=True)
    assert np.abs(K - Kref).max() <= 1e-10 * np.abs(Kref).max()
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(Kref).max()


def _high_l_df_system():
    """two atoms; orbital shells s (2 primitives), p, d with two contracted functions, f
    (2 primitives) and g on each atom, so AO-pair blocks reach 10 x 10 and 9 x 9 (above one warp's
    32 lanes) as well as 1 x 1; auxiliary s, p, d, f, g with one primitive each"""
    b = M._Builder()
    atoms = [b.atom(1, (0.0, 0.0, 0.0)), b.atom(1, (0.3, -0.5, 1.4))]
    for a in atoms:
        b.shell(a, 0, [3.1, 0.7], [M.gto_norm(0, 3.1) * 0.4, M.gto_norm(0, 0.7) * 0.8])
        b.shell(a, 1, [1.2], [M.gto_norm(1, 1.2)])
        b.shell(a, 2, [2.0, 0.6], [[M.gto_norm(2, 2.0) * 0.7, M.gto_norm(2, 0.6) * 0.5],
                                   [M.gto_norm(2, 2.0) * -0.3, M.gto_norm(2, 0.6) * 0.9]], nctr=2)
        b.shell(a, 3, [1.5, 0.5], [M.gto_norm(3, 1.5) * 0.6, M.gto_norm(3, 0.5) * 0.6])
        b.shell(a, 4, [0.9], [M.gto_norm(4, 0.9)])
    norb = 10
    for a in atoms:
        for l, e in ((0, 1.7), (1, 1.1), (2, 0.9), (3, 0.8), (4, 0.7)):
            b.shell(a, l, [e], [M.gto_norm(l, e)])
    return b.mol('df high l'), norb


@pytest.mark.parametrize('subset', [False, True])
def test_df_kernels_match_dense_formulation(gpulib, oracle, subset):
    """the DF kernels (cintgpu_df_rho / cintgpu_df_j) against the per-element torch formulation
    (gathers and scatter-adds over the same packed buffer) on AO-pair blocks from 1 x 1 to
    10 x 10 (both kernel paths), for all orbital pairs and for every other pair; with all pairs,
    also rho and J against the oracle's dense fit"""
    import torch
    mol, norb = _high_l_df_system()
    pairs = None
    if subset:
        ii, jj = np.tril_indices(norb)
        pairs = np.stack([ii, jj], 1)[::2]
    fit = df.DFCoulomb(mol, norb, pairs=pairs, chunk=7)      # several int3c2e chunks
    n = fit.nao
    d = np.random.RandomState(9).normal(0, 0.2, (n, n))
    dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    pair_idx, aux_idx = fit.index_maps()
    items3, _ = df.df_items(norb, mol.nbas, fit.pairs)
    w = torch.as_tensor(df.fit_weights(items3, df._nsph(mol)), device='cuda')
    rho = fit.rho(dm)
    rho_ref = df.contract_rho(fit.T, w, pair_idx, aux_idx, dm, fit.naux)
    assert torch.abs(rho - rho_ref).max().item() <= 1e-13 * torch.abs(rho_ref).max().item()
    c = fit.coefficients(dm)
    loc = np.concatenate([[0], np.cumsum(df._nsph(mol))])
    diag = np.zeros((n, n), dtype=bool)
    for i in range(norb):
        diag[loc[i]:loc[i + 1], loc[i]:loc[i + 1]] = True
    inpairs = np.zeros((n, n), dtype=bool)
    for i, j in fit.pairs:
        inpairs[loc[i]:loc[i + 1], loc[j]:loc[j + 1]] = inpairs[loc[j]:loc[j + 1], loc[i]:loc[i + 1]] = True
    Jref = df.contract_j(fit.T, pair_idx, aux_idx, c, n, torch.as_tensor(diag, device='cuda'))
    J = fit.vj(dm)
    assert torch.abs(J - Jref).max().item() <= 1e-13 * torch.abs(Jref).max().item()
    assert not J.cpu().numpy()[~inpairs].any()                 # blocks of absent pairs stay zero
    assert torch.abs(J - J.T).max().item() <= 1e-14 * torch.abs(Jref).max().item()
    if not subset:
        _, _, rho_o, J_o = _dense_df(oracle, mol, norb, dm.cpu().numpy())
        assert np.abs(rho.cpu().numpy() - rho_o).max() <= 1e-12 * np.abs(rho_o).max()
        assert np.abs(J.cpu().numpy() - J_o).max() <= 1e-10 * np.abs(J_o).max()
    fit.close()
