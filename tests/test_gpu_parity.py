"""Parity of the CUDA path (through the C-ABI) with the CPU oracle and libcint's golden values.

Tolerances: the reference's own accuracy statement is ~1e-12 relative (libcint README.rst:217)
and its root fits deviate from 60-digit values by up to ~4e-12 (n = 7), so element-wise gates are
ABS_TOL = 1e-12 absolute everywhere and REL_TOL = 1e-10 relative (plus BLOCK_TOL = 1e-13 of the
block's Cartesian maximum, the rounding every element of a transformed block carries) where
|ref| > 1e-10 and |ref| > 1e-3 * max|Cartesian block| (elements produced by cancellation in the
horizontal or cart -> sph transforms carry the block's absolute error, not their own relative
one; see assert_block_close).  Golden sums use libcint's own criterion
round(|v - ref| / sqrt(count), place) == 0 (testsuite/test_cint.py:148-149).
"""
import numpy as np
import pytest

from libcint_gb300 import molecules as M

pytestmark = pytest.mark.gpu

ABS_TOL = 1e-12
REL_TOL = 1e-10
BLOCK_TOL = 1e-13


def close_kat(v, ref, count, place):
    return round(abs(v - ref) / count ** .5, place) == 0


def assert_block_close(a, b, what='', scale=None):
    """abs <= ABS_TOL everywhere; |a - b| <= REL_TOL |b| + BLOCK_TOL scale where |b| > 1e-10 and
    the element is not dominated by cancellation, i.e. |b| > 1e-3 * scale (scale: the block's
    Cartesian maximum when given, else max|b|).  Cart -> sph of high-l shells cancels up to 5
    decades (an (ss|g) block has Cartesian elements 1e5 x its spherical ones) and the horizontal
    transfer (ij| = (i+1,j-1| + AB (i,j-1| cancels as well, so relative agreement of the cancelled
    elements is bounded by the conditioning, for libcint itself as well: elements below 1e-3 of
    the block's largest Cartesian element carry ~1e-14 of that maximum as rounding, i.e. up to
    ~1e-10 of themselves (libcint vs the oracle: 2.1e-10 at 1.1e-4 of the maximum)."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    d = np.abs(a - b)
    assert d.max(initial=0) <= ABS_TOL, '%s max abs diff %.3e' % (what, d.max(initial=0))
    sc = np.abs(b).max(initial=0) if scale is None else scale
    big = (np.abs(b) > 1e-10) & (np.abs(b) > 1e-3 * sc)
    if big.any():
        excess = (d[big] - BLOCK_TOL * sc) / np.abs(b[big])
        rel = excess.max()
        assert rel <= REL_TOL, '%s max rel diff beyond %.0e of the block scale: %.3e' % (
            what, BLOCK_TOL, rel)


def cart_scale(oracle, name, mol, q, nbas=None):
    """max |Cartesian block| of the same shells, the conditioning scale of a spherical block"""
    if not name.endswith('_sph'):
        return None
    _, c = oracle.port.call(name[:-4] + '_cart', mol, q, nbas=nbas)
    return np.abs(c).max(initial=0)


def test_rys_roots_match_oracle(gpulib, oracle):
    rng = np.random.RandomState(7)
    for n in range(1, gpulib.lib().cintgpu_rys_nmax() + 1):
        xs = np.concatenate([[0.0, 1e-14, 1e-7, 0.5, 1.0, 39.999, 40.0 + 5 * n, 1e3, 1e6],
                             rng.uniform(0, 60 + 5 * n, 40)])
        s, w = gpulib.rys_roots(n, xs)
        for i, x in enumerate(xs):
            so, wo = oracle.roots(n, x)
            f0 = wo.sum()
            assert np.abs(s[i] - so).max() < 1e-14, (n, x)
            assert np.abs(w[i] - wo).max() < 1e-14 * max(f0, 1e-300), (n, x)


def _kat_quartets():
    out = []
    for l in range(8):
        for k in range(l + 1):
            for j in range(8):
                for i in range(j + 1):
                    out.append((i, j, k, l))
    return out


@pytest.mark.parametrize('name,golden', [('int2e_sph', 56243.88080655417),
                                         ('int2e_ip1_sph', 115489.8647398112)])
def test_kat_dropin(gpulib, oracle, name, golden):
    """libcint testsuite/test_cint.py:479-480 through the drop-in (opt = NULL, nbas = 4)."""
    mol, nbas = M.kat_basis()
    v = 0.0
    cnt = 0
    worst = 0.0
    for q in _kat_quartets():
        flag, blk = gpulib.dropin(name, mol, q, nbas=nbas)
        oflag, oblk = oracle.port.call(name, mol, q, nbas=nbas)
        assert flag == oflag, q
        assert_block_close(blk, oblk, '%s %s' % (name, q), cart_scale(oracle, name, mol, q, nbas))
        worst = max(worst, np.abs(blk - oblk).max())
        v += np.abs(blk).sum()
        cnt += blk.size
    assert close_kat(v, golden, cnt, 8), (v, golden)


def test_kat_3c2e(gpulib, oracle):
    """libcint testsuite/test_3c2e.py:303 golden sum and the 3c2e == 4c2e(fit) identity."""
    mol, nbas = M.kat_basis_3c2e()
    fit = 8
    v, cnt = 0.0, 0
    for k in range(nbas):
        mol.bas[fit, M.ATOM_OF] = mol.bas[k, M.ATOM_OF]
        for j in range(nbas):
            for i in range(nbas):
                _, blk = gpulib.dropin('int3c2e_sph', mol, (i, j, k), nbas=nbas)
                _, oblk = oracle.port.call('int3c2e_sph', mol, (i, j, k), nbas=nbas)
                assert_block_close(blk, oblk, '3c2e %d %d %d' % (i, j, k),
                                   cart_scale(oracle, 'int3c2e_sph', mol, (i, j, k), nbas))
                _, b4 = gpulib.dropin('int2e_sph', mol, (i, j, k, fit), nbas=nbas)
                np.testing.assert_allclose(blk.ravel(), b4.ravel(), rtol=1e-10, atol=1e-12)
                v += np.abs(blk).sum()
                cnt += blk.size
    assert close_kat(v, 1586.350797347553, cnt, 10), v


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_cart', 'int2e_ip1_sph', 'int2e_ip1_cart'])
def test_config0_sample_dropin(gpulib, oracle, name):
    mol = M.config0(seed=3)
    rng = np.random.RandomState(1)
    qs = M.unique_quartets(mol.nbas)
    for q in qs[rng.choice(len(qs), 25, replace=False)]:
        flag, blk = gpulib.dropin(name, mol, q)
        oflag, oblk = oracle.port.call(name, mol, q)
        assert flag == oflag
        assert_block_close(blk, oblk, '%s %s' % (name, q), cart_scale(oracle, name, mol, q))


def test_dims_layout(gpulib, oracle):
    """dims gives the leading dimensions of a larger output (libcint src/cart2sph.c:5339-5342)."""
    mol = M.config0(seed=4)
    q = np.array([4, 2, 9, 3], dtype=np.int32)
    cnt = [mol.nsph(s) for s in q]
    dims = [c + 2 for c in cnt]
    _, out = gpulib.dropin('int2e_sph', mol, q, dims=dims)
    _, ref = oracle.port.call('int2e_sph', mol, q, dims=dims)
    assert_block_close(out, ref, 'dims', cart_scale(oracle, 'int2e_sph', mol, q))


@pytest.mark.parametrize('kind,name', [(1, 'int2e_sph'), (2, 'int2e_cart'), (3, 'int2e_ip1_sph')])
def test_batched_plan_config0(gpulib, oracle, kind, name):
    import torch
    mol = M.config0(seed=5)
    rng = np.random.RandomState(2)
    qs = M.unique_quartets(mol.nbas)
    qs = qs[rng.choice(len(qs), 300, replace=False)]
    p = gpulib.Plan(kind, mol, qs)
    out = torch.zeros(p.ncomp * p.output_size, dtype=torch.float64, device='cuda')
    p.execute(out)
    torch.cuda.synchronize()
    res = out.cpu().numpy().reshape(p.ncomp, p.output_size)
    off = 0
    for q in qs:
        _, oblk = oracle.port.call(name, mol, q)
        nb = oblk.size // p.ncomp
        got = res[:, off:off + nb]
        want = oblk.reshape(nb, p.ncomp, order='F').T if p.ncomp > 1 else oblk.reshape(1, nb, order='F')
        assert_block_close(got, want, '%s %s' % (name, q), cart_scale(oracle, name, mol, q))
        off += nb


def test_batched_3c2e(gpulib, oracle):
    import torch
    mol, norb = M.config2(seed=1, natm=6, box=5.0)
    rng = np.random.RandomState(3)
    items = []
    for _ in range(200):
        i, j = sorted(rng.randint(0, norb, 2))[::-1]
        k = rng.randint(norb, mol.nbas)
        items.append((i, j, k))
    items = np.array(items, dtype=np.int32)
    p = gpulib.Plan(gpulib.INT3C2E_SPH, mol, items)
    out = torch.zeros(p.output_size, dtype=torch.float64, device='cuda')
    p.execute(out)
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    off = 0
    for it in items:
        _, oblk = oracle.port.call('int3c2e_sph', mol, it)
        nb = oblk.size
        assert_block_close(res[off:off + nb], oblk.ravel(order='F'), '3c2e %s' % (it,),
                           cart_scale(oracle, 'int3c2e_sph', mol, it))
        off += nb


@pytest.mark.parametrize('key', ['kat_int2e_sph', 'kat_int2e_ip1_sph', 'c0_int2e_sph',
                                 'c0_int2e_cart', 'c0_int2e_ip1_sph', 'c2_int3c2e_sph'])
def test_gpu_matches_libcint_blocks(gpulib, oracle, key):
    """Directly against libcint's own output (tests/golden/ref_blocks.npz, generated by
    make_ref_blocks.py from libcint built from its sources)."""
    import os
    fx = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'ref_blocks.npz'))
    items, ref = fx[key + '_items'], fx[key]
    name = key.split('_', 1)[1]
    nbas = None
    if key.startswith('kat'):
        mol, nbas = M.kat_basis()
    elif key.startswith('c0'):
        mol = M.config0(seed=3)
    else:
        mol, _ = M.config2(seed=1, natm=6, box=5.0)
    off = 0
    for it in items:
        _, blk = gpulib.dropin(name, mol, it, nbas=nbas)
        b = blk.ravel(order='F')
        assert_block_close(b, ref[off:off + b.size], '%s %s' % (key, it),
                           cart_scale(oracle, name, mol, it, nbas))
        off += b.size
    assert off == ref.size
