"""int2c2e (i|k), the density-fitting metric, on the GPU: the drop-in (libcint signature, with and
without dims), batched plans and the host-buffer form, against the oracle, against libcint's own
blocks (golden fixture) and through the identity (i|k) = int3c2e(i, s0, k) with a zero-exponent
unit s shell.

Tolerance: the bars of the other parity tests on blocks scaled by 1 / max(1, Cartesian block
scale): two-centre blocks of diffuse normalised functions reach ~150, where 1e-12 absolute would be
below the ulp (libcint and the oracle differ by up to 3e-12 there, 2e-14 relative)."""
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests.test_gpu_parity import assert_block_close

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), 'golden')


def _close(got, ref, what, cart_max):
    s = max(1.0, cart_max)
    assert_block_close(np.asarray(got) / s, np.asarray(ref) / s, what, cart_max / s)


def _pairs(mol, n, seed):
    rng = np.random.RandomState(seed)
    return [(int(a), int(b)) for a, b in rng.randint(0, mol.nbas, (n, 2))]


def _mols():
    c2, _ = M.config2(seed=1, natm=4, box=4.0)
    kat, nk = M.kat_basis()
    return [(c2, _pairs(c2, 80, 0), None),
            (kat, [(i, k) for k in range(8) for i in range(8)], nk)]


@pytest.mark.parametrize('name', ['int2c2e_sph', 'int2c2e_cart'])
def test_2c2e_dropin_matches_oracle(gpulib, oracle, name):
    for mol, items, nb in _mols():
        for it in items:
            fo, ref = oracle.port.call(name, mol, it, nbas=nb)
            fg, got = gpulib.dropin(name, mol, it, nbas=nb)
            assert fo == fg
            _, c = oracle.port.call('int2c2e_cart', mol, it, nbas=nb)
            _close(got, ref, '%s %s' % (name, it), np.abs(c).max(initial=0))


def test_2c2e_dropin_dims(gpulib, oracle):
    """dims holds two leading dimensions; the rest of the caller's buffer stays untouched"""
    mol, items, _ = _mols()[0]
    for it in items[:10]:
        _, ref = oracle.port.call('int2c2e_sph', mol, it)
        dims = (ref.shape[0] + 3, ref.shape[1] + 2)
        _, got = gpulib.dropin('int2c2e_sph', mol, it, dims=dims)
        _, want = oracle.port.call('int2c2e_sph', mol, it, dims=dims)
        got = np.asarray(got).reshape(dims, order='F')
        want = np.asarray(want).reshape(dims, order='F')
        assert not got[ref.shape[0]:, :].any() and not got[:, ref.shape[1]:].any()
        _, c = oracle.port.call('int2c2e_cart', mol, it)
        _close(got, want, 'dims %s' % (it,), np.abs(c).max(initial=0))


@pytest.mark.parametrize('kind', ['INT2C2E_SPH', 'INT2C2E_CART'])
def test_2c2e_plan_and_batch_host(gpulib, oracle, kind):
    import torch
    name = kind.lower()
    for mol, items, nb in _mols():
        if nb is not None:
            continue   # plans take the whole basis
        plan = gpulib.Plan(getattr(gpulib, kind), mol, np.array(items, np.int32))
        out = torch.zeros(plan.output_size, dtype=torch.float64, device='cuda')
        plan.execute(out)
        res = out.cpu().numpy()
        plan.close()
        # the host-buffer form plans the list in chunks (other slice sums): oracle-checked too
        host = gpulib.batch_host(getattr(gpulib, kind), mol, np.array(items, np.int32))[0]
        assert host.size == res.size
        off = 0
        for it in items:
            _, ref = oracle.port.call(name, mol, it)
            _, c = oracle.port.call('int2c2e_cart', mol, it)
            for got, what in ((res, 'plan'), (host, 'batch_host')):
                _close(got[off:off + ref.size], ref.ravel(order='F'), '%s %s' % (what, it),
                       np.abs(c).max(initial=0))
            off += ref.size
        assert off == res.size


def test_2c2e_golden_blocks_and_3c2e_identity(gpulib, oracle):
    """libcint's own blocks (fixture), and (i|k) = int3c2e(i, fit, k) with the KAT basis's
    zero-exponent fit shell moved onto i's atom"""
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    mol, _ = M.config2(seed=1, natm=6, box=5.0)
    items, ref = fx['c2_int2c2e_sph_items'], fx['c2_int2c2e_sph']
    off = 0
    for it in items:
        _, got = gpulib.dropin('int2c2e_sph', mol, it)
        got = np.asarray(got).ravel(order='F')
        _, c = oracle.port.call('int2c2e_cart', mol, it)
        _close(got, ref[off:off + got.size], 'golden %s' % (it,), np.abs(c).max(initial=0))
        off += got.size
    assert off == ref.size
    kat, nbas = M.kat_basis_3c2e()
    for k in range(nbas):
        for i in range(nbas):
            kat.bas[8, M.ATOM_OF] = kat.bas[i, M.ATOM_OF]
            _, b2 = gpulib.dropin('int2c2e_sph', kat, (i, k), nbas=nbas)
            _, b3 = gpulib.dropin('int3c2e_sph', kat, (i, 8, k), nbas=nbas)
            np.testing.assert_allclose(np.asarray(b2).ravel(), np.asarray(b3).ravel(), rtol=1e-10,
                                       atol=1e-12)
