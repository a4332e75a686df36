"""Parity on the other workloads' shapes, through batched plans and the drop-in, against libcint's
own blocks (tests/golden/ref_blocks.npz), the CPU restatement and its long-double referee:

  c3   24 atoms, s/p/d with 3-5 primitives (the adjoint's workload): int2e_sph and int2e_ip1_sph
  c4   g shells with 1-8 primitives (one quartet per kernel-order class, l <= 4): int2e_sph,
       int2e_cart and int2e_ip1_sph
  c2   int3c2e_cart (the int3c2e_sph path is covered elsewhere)
  CINT2  the 8-argument wrappers (cint2e_sph, ...) equal the 10-argument entries.
Gates as in test_gpu_c1_sweep: 1e-12 absolute everywhere; 1e-10 relative against the referee on
elements above 1e-3 (Cartesian) or 1e-2 (spherical) of the quartet's largest Cartesian element."""
import ctypes
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests import c1_sample
from tests.test_gpu_c1_sweep import ABS_TOL, CUTOFF, REL_TOL, class_errors, gpu_blocks

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')


def c4_mol():
    return M.config4(seed=2, natm=4, box=5.2)


def item_major(gpu, mol, items, name):
    """plan output (component-major: comp * output_size + block offset) -> per item, all
    components (libcint's per-call layout)"""
    sph = name.endswith('_sph')
    ncomp = 9 if '_ipip1' in name else (3 if ('_ip1' in name or '_ip2' in name) else 1)
    nsh = 3 if 'int3c2e' in name else 4
    per = np.array([mol.nsph(s) if sph else mol.ncart(s) for s in range(mol.nbas)], dtype=np.int64)
    size = np.prod(per[np.asarray(items)[:, :nsh]], axis=1)
    offs = np.concatenate([[0], np.cumsum(size)])
    S = int(offs[-1])
    out = np.empty(S * ncomp)
    pos = 0
    for q in range(len(items)):
        for c in range(ncomp):
            out[pos:pos + size[q]] = gpu[c * S + offs[q]:c * S + offs[q + 1]]
            pos += size[q]
    return out


def scales(oracle, mol, items, three=False):
    name = 'int3c2e_cart' if three else 'int2e_cart'
    cart, offs = oracle.blocks(name, mol, items)
    return np.array([np.abs(cart[offs[q]:offs[q + 1]]).max(initial=0) for q in range(len(items))])


def check(gpu, ref, offs, cs, cls, name, what):
    d = np.abs(gpu - ref)
    assert d.max() <= ABS_TOL, '%s: max abs %.3e' % (what, d.max())
    per = class_errors(gpu, ref, offs, cs, cls, CUTOFF['int2e_sph' if name.endswith('_sph') else 'int2e_cart'])
    bad = {k: v for k, v in per.items() if v[1] > REL_TOL}
    assert not bad, (what, {k: '%.2e' % v[1] for k, v in sorted(bad.items())})


def no_worse_than_libcint(gpu, ref, offs, liberr, librel, cutoff, items, what, factor=10.0,
                          scale=None, rel_floor=1e-10):
    """Item by item against the long-double referee: the GPU's largest absolute error at most
    `factor` x libcint's own (or 2e-12), its largest relative error on elements above 1e-10 and
    above `cutoff` x the item's scale (the largest Cartesian element for spherical blocks) at
    most `factor` x libcint's (or 1e-10); and the worst absolute error over all items at most
    3 x libcint's worst."""
    from tests.golden.make_ref_blocks import item_errors
    ea, er = item_errors(gpu, ref, offs, cutoff, scale)
    bad = [(items[q].tolist(), '%.2e/%.2e' % (ea[q], er[q]), '%.2e/%.2e' % (liberr[q], librel[q]))
           for q in range(len(ea))
           if ea[q] > max(2e-12, factor * liberr[q]) or er[q] > max(rel_floor, factor * librel[q])]
    assert not bad, (what, bad[:8])
    assert ea.max() <= max(2e-12, 3 * liberr.max()), (what, ea.max(), liberr.max())


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_cart', 'int2e_ip1_sph'])
def test_c4_g_shell_classes(gpulib, oracle, name):
    """g shells on a dense 4-atom geometry, one quartet per class: the ill-conditioned end of the
    transfers, where libcint itself is up to 1.1e-11 absolute and 2e-8 relative off the referee
    (tests/golden/ref_blocks.npz records libcint's errors per quartet); the bar is libcint's own
    accuracy quartet by quartet (10x, with floors of 2e-12 absolute and 2e-10 relative: one
    (gg|gd) nabla element of this geometry sits at 1.6e-10 against libcint's 3.7e-12)."""
    mol = c4_mol()
    from tests.golden.make_ref_blocks import c4_class_quartets
    qs = c4_class_quartets(mol)
    assert len(qs) == 120 and c1_sample.kernel_class(mol, qs).max() == 4
    gpu = item_major(gpu_blocks(gpulib, name, mol, qs), mol, qs, name)
    ref, offs = oracle.referee(name, mol, qs)
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    key = 'c4_' + name
    np.testing.assert_array_equal(fx[key + '_items'], qs)
    from tests.golden.make_ref_blocks import cart_scale
    no_worse_than_libcint(gpu, ref, offs, fx[key + '_liberr'], fx[key + '_librel'],
                          1e-2 if name.endswith('_sph') else 1e-3, qs, key,
                          scale=cart_scale(oracle, name, mol, qs), rel_floor=2e-10)
    assert np.abs(gpu - fx[key]).max() <= 3 * fx[key + '_liberr'].max() + 2e-12


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_ip1_sph'])
def test_c3_blocks(gpulib, oracle, name):
    """c3: a class-stratified sample of the full unique list (plans) and libcint's own 40 blocks
    (drop-in)."""
    mol = M.config3(seed=0)
    allq = M.unique_quartets(mol.nbas)
    allq = allq[np.random.RandomState(11).permutation(len(allq))]
    qs, cls = c1_sample.stratified(mol, allq, 40)
    gpu = item_major(gpu_blocks(gpulib, name, mol, qs), mol, qs, name)
    ref, offs = oracle.referee(name, mol, qs)
    check(gpu, ref, offs, scales(oracle, mol, qs), cls, name, 'c3 %s vs referee' % name)
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    items, lib = fx['c3_' + name + '_items'], fx['c3_' + name]
    off = 0
    for it in items:
        _, blk = gpulib.dropin(name, mol, it)
        b = blk.ravel(order='F')
        assert np.abs(b - lib[off:off + b.size]).max() <= ABS_TOL, it
        off += b.size
    assert off == lib.size


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_cart'])
def test_c1_libcint_blocks(gpulib, oracle, name):
    """The benchmark workload's classes against libcint's own blocks: 2 quartets per class."""
    mol = M.config1(seed=0)
    fx = np.load(os.path.join(GOLD, 'ref_blocks.npz'))
    qs, lib = fx['c1_' + name + '_items'], fx['c1_' + name]
    gpu = gpu_blocks(gpulib, name, mol, qs)
    assert gpu.size == lib.size
    assert np.abs(gpu - lib).max() <= ABS_TOL


def test_int3c2e_cart(gpulib, oracle):
    mol, norb = M.config2(seed=1, natm=6, box=5.0)
    rng = np.random.RandomState(4)
    tr = []
    for _ in range(300):
        i, j = sorted(rng.randint(0, norb, 2))[::-1]
        tr.append((i, j, rng.randint(norb, mol.nbas)))
    tr = np.array(tr, dtype=np.int32)
    gpu = gpu_blocks(gpulib, 'int3c2e_cart', mol, tr)
    ref, offs = oracle.referee('int3c2e_cart', mol, tr)
    cs = np.array([np.abs(ref[offs[q]:offs[q + 1]]).max(initial=0) for q in range(len(tr))])
    L = mol.bas[:, 1]
    cls = np.stack([L[tr[:, 0]], L[tr[:, 1]], L[tr[:, 2]], 0 * tr[:, 0]], 1)
    check(gpu, ref, offs, cs, cls, 'int3c2e_cart', 'int3c2e_cart vs referee')
    for t in tr[:20]:
        _, blk = gpulib.dropin('int3c2e_cart', mol, t)
        _, o = oracle.port.call('int3c2e_cart', mol, t)
        assert np.abs(blk - o).max() <= ABS_TOL


@pytest.mark.parametrize('name,nsh', [('cint2e_sph', 4), ('cint2e_cart', 4), ('cint2e_ip1_sph', 4),
                                      ('cint2e_ip1_cart', 4), ('cint3c2e_sph', 3),
                                      ('cint3c2e_cart', 3), ('cint2c2e_sph', 2), ('cint2c2e_cart', 2)])
def test_cint2_wrappers(gpulib, name, nsh):
    """libcint's 8-argument CINT2 forms (src/misc.h:34-60) give the 10-argument entries' blocks
    and return value, with and without an optimizer."""
    L = gpulib.lib()
    mol, norb = M.config2(seed=1, natm=4, box=4.0)
    P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)
    rng = np.random.RandomState(nsh)
    opt = ctypes.c_void_p()
    optf = {'cint2e_sph': 'cint2e_sph_optimizer', 'cint2e_ip1_sph': 'cint2e_ip1_sph_optimizer',
            'cint3c2e_sph': 'cint3c2e_sph_optimizer', 'cint2c2e_sph': 'cint2c2e_sph_optimizer'}.get(name)
    if optf:
        getattr(L, optf)(ctypes.byref(opt), P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env))
    for _ in range(6):
        s = np.ascontiguousarray(rng.randint(0, mol.nbas, 4), dtype=np.int32)
        flag10, ref = gpulib.dropin(name[1:], mol, s[:nsh])
        out = np.zeros(ref.size)
        f = getattr(L, name)
        flag8 = f(P(out), P(s), P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env), opt)
        assert flag8 == flag10
        np.testing.assert_array_equal(out, ref.ravel(order='F'))
    if optf:
        L.CINTdel_optimizer(ctypes.byref(opt))


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_ip1_sph', 'int3c2e_sph'])
def test_dropin_flags_sparse(gpulib, oracle, name):
    """the drop-in's return value on a sparse system where about 40 % of the quartets (15 % of
    the triples) have every primitive screened out: the oracle's flag (pinned to libcint's by
    test_oracle_flags_match_libcint_sparse), a zero block for 0, the oracle's block for 1, with
    and without an optimizer"""
    from tests.test_oracle import sparse_items
    mol, q4, q3 = sparse_items()
    items = q3 if name == 'int3c2e_sph' else (q4[:150] if '_ip1' in name else q4)
    L = gpulib.lib()
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    opt = ctypes.c_void_p()
    optf = 'int3c2e_optimizer' if name == 'int3c2e_sph' else ('int2e_ip1_optimizer' if '_ip1' in name
                                                             else 'int2e_optimizer')
    getattr(L, optf)(ctypes.byref(opt), P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env))
    f = getattr(L, name)
    flags = []
    try:
        for it in items:
            s = np.ascontiguousarray(it, dtype=np.int32)
            fo, ref = oracle.port.call(name, mol, s)
            for o in (None, opt):
                out = np.full(ref.size, 7.0)
                fg = f(P(out), None, P(s), P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env),
                       o, None)
                assert fg == fo
                if fo == 0:
                    assert not out.any()
                else:
                    assert np.abs(out - ref.ravel(order='F')).max() <= ABS_TOL
            flags.append(fo)
    finally:
        L.CINTdel_optimizer(ctypes.byref(opt))
    assert set(flags) == {0, 1}
