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
