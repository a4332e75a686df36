"""Long-range Coulomb erf(omega r)/r (env[PTR_RANGE_OMEGA] = omega > 0; libcint src/g2e.c:4477-4492):
the oracle's restatement against libcint's own blocks (tests/golden/ref_blocks.npz), live libcint
where it is built here, and the identity that it is the full Coulomb in the limit omega -> inf and
vanishes as omega -> 0.  CPU only; the GPU path is in test_gpu_range_separated.py."""
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M

GOLD = os.path.join(os.path.dirname(__file__), 'golden')


def lr_mol(which, short_range=False):
    """the fixture molecules: c0(3) with omega 0.3, the c2 molecule with 0.5 (negative: the
    short-range operator)"""
    if which == 'c0':
        mol = M.config0(seed=3)
        mol.env[8] = 0.3                       # PTR_RANGE_OMEGA
    else:
        mol, _ = M.config2(seed=1, natm=6, box=5.0)
        mol.env[8] = 0.5
    if short_range:
        mol.env[8] = -mol.env[8]
    return mol


RS_KEYS = [p + k for p in ('lr_', 'sr_') for k in ('c0_int2e_sph', 'c0_int2e_ip1_sph',
                                                   'c2_int3c2e_sph', 'c2_int2c2e_sph')]


@pytest.mark.parametrize('key', RS_KEYS)
def test_oracle_lr_matches_libcint_blocks(oracle, key):
    """long range (lr_) and short range (sr_: the oracle's own roots of the erfc-weighted
    quadrature, libcint's full-minus-long-range or SR root finders) against libcint's blocks"""
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    items, ref = fx[key + '_items'], fx[key]
    name = key.split('_', 2)[2]
    mol = lr_mol(key.split('_')[1], key.startswith('sr_'))
    got, offs = oracle.blocks(name, mol, items)
    scale = np.abs(ref).max()
    atol = 1e-12 * max(1.0, scale) if '2c2e' in name else 1e-12
    assert np.abs(got - ref).max() <= atol


def test_lr_limits(oracle):
    mol = M.config0(seed=3)
    q = np.array([[7, 3, 5, 1]], np.int32)
    full, _ = oracle.blocks('int2e_sph', mol, q)
    mol.env[8] = 1e8
    big, _ = oracle.blocks('int2e_sph', mol, q)
    mol.env[8] = 1e-6
    small, _ = oracle.blocks('int2e_sph', mol, q)
    assert np.abs(big - full).max() <= 1e-12 * np.abs(full).max()
    assert np.abs(small).max() <= 1e-5 * np.abs(full).max()


def test_short_plus_long_range_is_coulomb(oracle):
    """erfc(wr)/r + erf(wr)/r = 1/r, element by element, for int2e (c0 quartets with s..d shells),
    int2e_ip1 and int3c2e, at three omegas"""
    mol = M.config0(seed=3)
    q = np.asarray(M.unique_quartets(mol.nbas))[::41][:80]
    for name in ('int2e_sph', 'int2e_ip1_sph'):
        full, _ = oracle.blocks(name, mol, q)
        for w in (0.1, 0.5, 2.0):
            m = mol.copy()
            m.env[8] = w
            lr, _ = oracle.blocks(name, m, q)
            m.env[8] = -w
            sr, _ = oracle.blocks(name, m, q)
            assert np.abs(sr + lr - full).max() <= 1e-12 * np.abs(full).max(), (name, w)
            assert np.abs(sr).max() > 1e-3 * np.abs(full).max()
