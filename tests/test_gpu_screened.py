"""Whole-molecule Schwarz-screened J / K / adjoint (cintgpu_screened_run through
screening.ScreenedCoulomb): the streamed list is exactly the explicit screened list, its J, K and
gradient equal those of plans over that explicit list, slabs of bra pairs add up to the whole, and
a zero threshold reproduces the full unique list."""
import numpy as np
import pytest

from libcint_gb300 import molecules as M

pytestmark = pytest.mark.gpu


def _dm(mol, seed=0):
    import torch
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    d = np.random.RandomState(seed).normal(0, 0.1, (nao, nao))
    return torch.as_tensor(0.5 * (d + d.T), device='cuda')


def test_screened_matches_explicit_list(gpulib):
    import torch
    from libcint_gb300.coulomb import CoulombPlans
    from libcint_gb300.screening import ScreenedCoulomb, screened_list
    mol = M.config3(seed=1, natm=8, box=8.0 * (8 / 24) ** (1 / 3) * 1.6)
    dm = _dm(mol)
    sc = ScreenedCoulomb(mol, threshold=1e-9)
    J, K = sc.get_jk(dm)
    nq = sc.last_quartets
    lst = screened_list(sc.q, sc.pairs, 1e-9)
    assert nq == len(lst)
    full = len(M.unique_quartets(mol.nbas))
    assert 0 < nq < full                       # the screening removed something
    ref = CoulombPlans(mol, lst)
    J0, K0 = ref.get_jk(dm)
    assert float((J - J0).abs().max()) <= 1e-11 * float(J0.abs().max())
    assert float((K - K0).abs().max()) <= 1e-11 * float(K0.abs().max())
    g, _ = sc.grad(dm)
    g0, _ = ref.grad(dm)
    assert float((g - g0).abs().max()) <= 1e-11 * float(g0.abs().max())
    # two slabs of bra positions add up to the whole
    npair = len(sc.pairs)
    Ja, _ = sc.get_jk(dm, True, False, bra_range=(0, npair // 3))
    na = sc.last_quartets
    Jb, _ = sc.get_jk(dm, True, False, bra_range=(npair // 3, npair))
    assert na + sc.last_quartets == nq
    assert float((Ja + Jb - J).abs().max()) <= 1e-11 * float(J.abs().max())


def test_screened_zero_threshold_is_the_full_list(gpulib):
    from libcint_gb300.coulomb import CoulombPlans
    from libcint_gb300.screening import ScreenedCoulomb
    mol = M.config0(seed=2)
    dm = _dm(mol, 1)
    sc = ScreenedCoulomb(mol, threshold=0.0)
    J, K = sc.get_jk(dm)
    assert sc.last_quartets == len(M.unique_quartets(mol.nbas))
    J0, K0 = CoulombPlans(mol).get_jk(dm)
    assert float((J - J0).abs().max()) <= 1e-11 * float(J0.abs().max())
    assert float((K - K0).abs().max()) <= 1e-11 * float(K0.abs().max())
