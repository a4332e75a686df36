"""Long-range Coulomb erf(omega r)/r (env[PTR_RANGE_OMEGA] = omega > 0; libcint src/g2e.c:4477-4492):
the oracle's restatement against libcint's own blocks (tests/golden/ref_blocks.npz), live libcint
where it is built here, and the identity that it is the full Coulomb in the limit omega -> inf and
vanishes as omega -> 0.  CPU only; the GPU path is in test_gpu_range_separated.py."""
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M

GOLD = os.path.join(os.path.dirname(__file__), 'golden')


def lr_mol(which):
    if which == 'c0':
        mol = M.config0(seed=3)
        mol.env[8] = 0.3                       # PTR_RANGE_OMEGA
        return mol
    mol, _ = M.config2(seed=1, natm=6, box=5.0)
    mol.env[8] = 0.5
    return mol


@pytest.mark.parametrize('key', ['lr_c0_int2e_sph', 'lr_c0_int2e_ip1_sph', 'lr_c2_int3c2e_sph',
                                 'lr_c2_int2c2e_sph'])
def test_oracle_lr_matches_libcint_blocks(oracle, key):
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    items, ref = fx[key + '_items'], fx[key]
    name = key.split('_', 2)[2]
    mol = lr_mol(key.split('_')[1])
    assert mol.env[8] > 0
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
