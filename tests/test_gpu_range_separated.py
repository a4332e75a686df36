"""Range-separated Coulomb on the GPU (plans and the drop-in): the long-range erf(omega r)/r
(omega > 0) and the short-range erfc(omega r)/r (omega < 0) against the oracle and libcint's own
blocks for int2e_sph, int2e_ip1_sph, int3c2e_sph and int2c2e_sph, and short + long range = the
Coulomb operator on the GPU itself."""
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests.test_gpu_c1_sweep import ABS_TOL, gpu_blocks
from tests.test_gpu_configs import item_major
from tests.test_range_separated import RS_KEYS, lr_mol

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')


@pytest.mark.parametrize('key', RS_KEYS)
def test_gpu_lr_matches_libcint_blocks(gpulib, key):
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    items, ref = fx[key + '_items'], fx[key]
    name = key.split('_', 2)[2]
    mol = lr_mol(key.split('_')[1], key.startswith('sr_'))
    atol = ABS_TOL * max(1.0, np.abs(ref).max()) if '2c2e' in name else ABS_TOL
    off = 0
    for it in items:
        _, blk = gpulib.dropin(name, mol, it)
        b = blk.ravel(order='F')
        assert np.abs(b - ref[off:off + b.size]).max() <= atol, (key, it)
        off += b.size
    if name in ('int2e_sph', 'int2e_ip1_sph', 'int3c2e_sph'):
        gpu = item_major(gpu_blocks(gpulib, name, mol, items), mol, items, name)
        assert np.abs(gpu - ref).max() <= atol


def test_gpu_lr_c1_sample(gpulib, oracle):
    """Batched plans over 2000 quartets of the benchmark list with omega = 0.4."""
    from tests import c1_sample
    mol = M.config1(seed=0)
    mol.env[8] = 0.4
    qs = c1_sample.c1_quartets()[:2000]
    ref, offs = oracle.blocks('int2e_sph', mol, qs)
    got = gpu_blocks(gpulib, 'int2e_sph', mol, qs)
    assert np.abs(got - ref).max() <= ABS_TOL
    mol.env[8] = 0.0
    full = gpu_blocks(gpulib, 'int2e_sph', mol, qs)
    assert np.abs(full - got).max() > 1e-6      # the attenuation is really applied


def test_gpu_sr_c1_sample(gpulib, oracle):
    """Batched plans over 2000 quartets of the benchmark list with omega = -0.4 against the
    oracle (its own roots of the erfc-weighted quadrature), and short + long range = Coulomb."""
    from tests import c1_sample
    mol = M.config1(seed=0)
    qs = c1_sample.c1_quartets()[:2000]
    full = gpu_blocks(gpulib, 'int2e_sph', mol, qs)
    mol.env[8] = -0.4
    ref, offs = oracle.blocks('int2e_sph', mol, qs)
    sr = gpu_blocks(gpulib, 'int2e_sph', mol, qs)
    assert np.abs(sr - ref).max() <= ABS_TOL
    mol.env[8] = 0.4
    lr = gpu_blocks(gpulib, 'int2e_sph', mol, qs)
    assert np.abs(sr + lr - full).max() <= ABS_TOL
    assert np.abs(sr).max() > 1e-3 * np.abs(full).max()
