"""The derivative family on the GPU: (ij|nabla k l) (int2e_ip2), (nabla i j|k) (int3c2e_ip1),
(ij|nabla k) (int3c2e_ip2) and (nabla nabla i j|k l) (int2e_ipip1), sph and cart, through batched plans and the drop-in, against libcint's
own blocks (tests/golden/ref_blocks.npz), the restatement and its long-double referee; plus the
translational-invariance identity of the 3c2e derivatives:
(nabla_i j|k) + (i nabla_j|k) + (ij|nabla_k) = 0, with (i nabla_j|k) from int3c2e_ip1 of (j, i, k)."""
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests.test_gpu_c1_sweep import ABS_TOL, gpu_blocks
from tests.test_gpu_configs import item_major, no_worse_than_libcint

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')


def _mol(key):
    if key.startswith('c0'):
        return M.config0(seed=3)
    mol, _ = M.config2(seed=1, natm=6, box=5.0)
    return mol


@pytest.mark.parametrize('key', ['c0_int2e_ip2_sph', 'c0_int2e_ip2_cart', 'c2_int3c2e_ip1_sph',
                                 'c2_int3c2e_ip1_cart', 'c2_int3c2e_ip2_sph', 'c2_int3c2e_ip2_cart',
                                 'c0_int2e_ipip1_sph', 'c0_int2e_ipip1_cart'])
def test_derivatives_match_libcint(gpulib, oracle, key):
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    items, ref = fx[key + '_items'], fx[key]
    name = key.split('_', 1)[1]
    mol = _mol(key)
    gpu = item_major(gpu_blocks(gpulib, name, mol, items), mol, items, name)
    assert gpu.size == ref.size
    assert np.abs(gpu - ref).max() <= ABS_TOL, np.abs(gpu - ref).max()
    off = 0
    for it in items[:15]:
        _, blk = gpulib.dropin(name, mol, it)
        b = blk.ravel(order='F')
        assert np.abs(b - ref[off:off + b.size]).max() <= ABS_TOL
        off += b.size
    # against the referee, item by item no worse than libcint's own accuracy (libcint is up to
    # 2e-8 relative off on some (nabla i j|k) elements of this geometry)
    rf, offs = oracle.referee(name, mol, items)
    from tests.golden.make_ref_blocks import cart_scale
    no_worse_than_libcint(gpu, rf, offs, fx[key + '_liberr'], fx[key + '_librel'],
                          1e-2 if name.endswith('_sph') else 1e-3, items, key,
                          scale=cart_scale(oracle, name, mol, items))


def test_int2e_ip2_c3_sample(gpulib, oracle):
    """1000 c3 quartets (s, p, d x 3-5 primitives) through one batched int2e_ip2_sph plan."""
    mol = M.config3(seed=0)
    qs = M.unique_quartets(mol.nbas)
    qs = qs[np.random.RandomState(5).choice(len(qs), 1000, replace=False)]
    gpu = item_major(gpu_blocks(gpulib, 'int2e_ip2_sph', mol, qs), mol, qs, 'int2e_ip2_sph')
    ref, _ = oracle.blocks('int2e_ip2_sph', mol, qs)
    assert np.abs(gpu - ref).max() <= ABS_TOL


def test_int2e_ipip1_c3_sample(gpulib, oracle):
    """500 c3 quartets through one batched int2e_ipip1_sph plan (9 components), and the symmetry
    of the second nabla (component xy = yx, xz = zx, yz = zy)."""
    mol = M.config3(seed=0)
    qs = M.unique_quartets(mol.nbas)
    qs = qs[np.random.RandomState(6).choice(len(qs), 500, replace=False)]
    raw = gpu_blocks(gpulib, 'int2e_ipip1_sph', mol, qs)
    gpu = item_major(raw, mol, qs, 'int2e_ipip1_sph')
    ref, _ = oracle.blocks('int2e_ipip1_sph', mol, qs)
    assert np.abs(gpu - ref).max() <= ABS_TOL * max(1.0, np.abs(ref).max())
    c = raw.reshape(9, -1)
    assert np.array_equal(c[1], c[3]) and np.array_equal(c[2], c[6]) and np.array_equal(c[5], c[7])


def test_int3c2e_translational_invariance(gpulib):
    mol, norb = M.config2(seed=1, natm=6, box=5.0)
    rng = np.random.RandomState(6)
    tr = np.array([(rng.randint(0, norb), rng.randint(0, norb), rng.randint(norb, mol.nbas))
                   for _ in range(200)], dtype=np.int32)
    tr_ji = np.ascontiguousarray(tr[:, [1, 0, 2]])
    a = item_major(gpu_blocks(gpulib, 'int3c2e_ip1_cart', mol, tr), mol, tr, 'int3c2e_ip1_cart')
    b = item_major(gpu_blocks(gpulib, 'int3c2e_ip1_cart', mol, tr_ji), mol, tr_ji, 'int3c2e_ip1_cart')
    c = item_major(gpu_blocks(gpulib, 'int3c2e_ip2_cart', mol, tr), mol, tr, 'int3c2e_ip2_cart')
    n = np.array([mol.ncart(s) for s in range(mol.nbas)])
    pos = 0
    worst = 0.0
    for t in range(len(tr)):
        ni, nj, nk = n[tr[t, 0]], n[tr[t, 1]], n[tr[t, 2]]
        sz = ni * nj * nk * 3
        A = a[pos:pos + sz].reshape(3, nk, nj, ni)
        B = b[pos:pos + sz].reshape(3, nk, ni, nj).transpose(0, 1, 3, 2)
        C = c[pos:pos + sz].reshape(3, nk, nj, ni)
        worst = max(worst, np.abs(A + B + C).max() / max(np.abs(A).max(), 1e-300))
        pos += sz
    assert worst < 1e-11, worst
