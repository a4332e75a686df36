"""Generate tests/golden/ref_blocks.npz: libcint's own output blocks for a fixed set of shell
quartets/triples, so the oracle and the CUDA path can be compared with the reference itself on
machines where libcint's sources (and so oracle/_ref/libcint.so) are absent.

Run where libcint's sources exist:  make -C oracle ref && python tests/golden/make_ref_blocks.py

Contents (all through libcint 6.1.1 built by oracle/Makefile, opt = NULL, cache = NULL):
  kat_int2e_sph / kat_int2e_ip1_sph  90 quartets (every 5th with <= 450 elements) of libcint
                                     testsuite/test_cint.py's loop over its self-contained basis
                                     (nbas = 4 passed, 8 shells)
  c0_int2e_sph / c0_int2e_cart / c0_int2e_ip1_sph   60 unique quartets of molecules.config0(3)
  c2_int3c2e_sph                     60 (ij|P) triples of molecules.config2(1, natm=6, box=5)
  c2_int2c2e_sph / c2_int2c2e_cart   60 (i|k) pairs of the same molecule (orbital and auxiliary)
  kat_int2c2e_sph                    all 8 x 8 shell pairs of the self-contained basis
  hl_int2e_sph / hl_int2e_cart / hl_int3c2e_sph / hl_int2e_ip1_sph
                                     small blocks of the l = 6 / 5 / 4 / 2 / 0 basis of
                                     tests/test_gpu_high_l.py (i, h with two columns, g, d, s)
  c1_int2e_sph / c1_int2e_cart       the first 2 quartets of every kernel-order class of the
                                     benchmark list (tests/golden/c1_quartets.npz; 110 quartets)
  c4_int2e_sph / _cart / _ip1_sph    one quartet per kernel-order class (l <= 4, g shells, 1-8
                                     primitives) of molecules.config4(seed=2, natm=4, box=5.2)
  *_liberr / *_librel                for the c4 and derivative keys: libcint's own largest absolute
                                     and relative error per item against the long-double build of
                                     the restatement
  c3_int2e_sph / c3_int2e_ip1_sph    40 unique quartets of molecules.config3(seed=0)
  c0_int2e_ip2_sph / _cart           40 of the c0 quartets above, (ij|nabla k l)
  c0_int2e_ipip1_sph / _cart         the same 40, (nabla nabla i j|k l), 9 components
  c2_int3c2e_ip1_sph / _cart, c2_int3c2e_ip2_sph / _cart    the 60 c2 triples above
  lr_c0_int2e_sph / lr_c0_int2e_ip1_sph / lr_c2_int3c2e_sph / lr_c2_int2c2e_sph
                                     long-range Coulomb erf(omega r)/r (env[PTR_RANGE_OMEGA] =
                                     0.3 for c0(3), 0.5 for the c2 molecule): 30 / 30 / 40 / 40 items
  sr_c0_* / sr_c2_*                  the same items with short-range Coulomb erfc(omega r)/r
                                     (env[PTR_RANGE_OMEGA] = -0.3, -0.5)
  cache_sizes                        the out == NULL cache-size answers for a few items
Each block is stored flattened in libcint's (Fortran) order with its item list.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libcint_gb300 import molecules as M  # noqa: E402
from tests import _oracle  # noqa: E402
from tests.test_gpu_high_l import high_l_basis  # noqa: E402

HL_ITEMS = {
    'int2e_sph': [(0, 4, 0, 3), (0, 0, 4, 4), (2, 1, 3, 4), (1, 4, 3, 4), (0, 3, 3, 4), (1, 2, 3, 4),
                  (0, 2, 4, 3), (1, 3, 1, 4), (0, 1, 3, 4)],
    'int2e_cart': [(0, 4, 0, 3), (0, 0, 4, 4), (2, 1, 3, 4), (1, 4, 3, 4), (0, 3, 3, 4), (1, 2, 3, 4)],
    'int3c2e_sph': [(3, 4, 0), (0, 3, 2), (1, 4, 2), (0, 0, 4)],
    'int2e_ip1_sph': [(1, 2, 3, 4), (0, 3, 4, 4), (2, 0, 3, 4)],
}


def item_errors(got, ref, offs, cutoff, scale=None):
    """per item: (largest absolute error, largest relative error on elements with |ref| > 1e-10
    and |ref| > cutoff x scale[q]; scale: the item's largest Cartesian element for spherical
    blocks, default the item's own largest |ref|)"""
    ea, er = np.zeros(len(offs) - 1), np.zeros(len(offs) - 1)
    for q in range(len(offs) - 1):
        a, b = got[offs[q]:offs[q + 1]], ref[offs[q]:offs[q + 1]]
        d = np.abs(a - b)
        ea[q] = d.max(initial=0)
        sc = np.abs(b).max(initial=0) if scale is None else scale[q]
        big = (np.abs(b) > 1e-10) & (np.abs(b) > cutoff * sc)
        er[q] = (d[big] / np.abs(b[big])).max(initial=0)
    return ea, er


def cart_scale(oracle, name, mol, items):
    """largest element of each item's Cartesian block (all components): the conditioning scale of
    a spherical block; None for Cartesian kinds"""
    if not name.endswith('_sph'):
        return None
    cart, offs = oracle.blocks(name[:-4] + '_cart', mol, items)
    return np.array([np.abs(cart[offs[q]:offs[q + 1]]).max(initial=0) for q in range(len(items))])


def c4_class_quartets(mol, seed=5):
    """One unique quartet per kernel-order class (li >= lj, lk >= ll, (li lj) >= (lk ll)) of mol,
    drawn with a fixed seed; the list every g-shell test uses."""
    from tests import c1_sample
    qs = M.unique_quartets(mol.nbas)
    rng = np.random.RandomState(seed)
    qs = qs[rng.permutation(len(qs))]
    k = c1_sample.kernel_class(mol, qs)
    key = ((k[:, 0] * 8 + k[:, 1]) * 8 + k[:, 2]) * 8 + k[:, 3]
    _, first = np.unique(key, return_index=True)
    return np.ascontiguousarray(qs[np.sort(first)], dtype=np.int32)


def main():
    o = _oracle.load()
    assert o.ref is not None, 'build libcint first: make -C oracle ref'
    out = {}
    mol, nbas = M.kat_basis()
    items = []
    for l in range(8):
        for k in range(l + 1):
            for j in range(8):
                for i in range(j + 1):
                    items.append((i, j, k, l))
    size = lambda q: int(np.prod([mol.nsph(s) for s in q]))
    items = np.array([q for q in items[::5] if size(q) <= 450][:90], dtype=np.int32)
    for name in ('int2e_sph', 'int2e_ip1_sph'):
        blocks = [o.ref.call(name, mol, q, nbas=nbas)[1].ravel(order='F') for q in items]
        out['kat_' + name + '_items'] = items
        out['kat_' + name] = np.concatenate(blocks)
    mol0 = M.config0(seed=3)
    rng = np.random.RandomState(9)
    qs = M.unique_quartets(mol0.nbas)
    qs = qs[rng.choice(len(qs), 60, replace=False)].astype(np.int32)
    for name in ('int2e_sph', 'int2e_cart', 'int2e_ip1_sph'):
        blocks = [o.ref.call(name, mol0, q)[1].ravel(order='F') for q in qs]
        out['c0_' + name + '_items'] = qs
        out['c0_' + name] = np.concatenate(blocks)
    mol2, norb = M.config2(seed=1, natm=6, box=5.0)
    tr = []
    for _ in range(60):
        i, j = sorted(rng.randint(0, norb, 2))[::-1]
        tr.append((i, j, rng.randint(norb, mol2.nbas)))
    tr = np.array(tr, dtype=np.int32)
    out['c2_int3c2e_sph_items'] = tr
    out['c2_int3c2e_sph'] = np.concatenate([o.ref.call('int3c2e_sph', mol2, t)[1].ravel(order='F')
                                            for t in tr])
    pr = np.array([(rng.randint(0, mol2.nbas), rng.randint(0, mol2.nbas)) for _ in range(60)],
                  dtype=np.int32)
    for name in ('int2c2e_sph', 'int2c2e_cart'):
        out['c2_' + name + '_items'] = pr
        out['c2_' + name] = np.concatenate([o.ref.call(name, mol2, t)[1].ravel(order='F') for t in pr])
    hl = high_l_basis()
    for name, items in HL_ITEMS.items():
        it = np.array(items, dtype=np.int32)
        out['hl_' + name + '_items'] = it
        out['hl_' + name] = np.concatenate([o.ref.call(name, hl, t)[1].ravel(order='F') for t in it])
    # the benchmark workload's classes (2 quartets of each, list order)
    from tests import c1_sample
    mol1 = M.config1(seed=0)
    q1, _ = c1_sample.stratified(mol1, c1_sample.c1_quartets(), 2)
    for name in ('int2e_sph', 'int2e_cart'):
        out['c1_' + name + '_items'] = q1
        out['c1_' + name] = np.concatenate([o.ref.call(name, mol1, q)[1].ravel(order='F') for q in q1])
    # g shells: one quartet per kernel-order class of a small c4-type molecule
    mol4 = M.config4(seed=2, natm=4, box=5.2)
    q4 = c4_class_quartets(mol4)
    for name in ('int2e_sph', 'int2e_cart', 'int2e_ip1_sph'):
        out['c4_' + name + '_items'] = q4
        out['c4_' + name] = np.concatenate([o.ref.call(name, mol4, q)[1].ravel(order='F') for q in q4])

    mol3 = M.config3(seed=0)
    q3 = M.unique_quartets(mol3.nbas)
    q3 = q3[np.random.RandomState(3).choice(len(q3), 40, replace=False)].astype(np.int32)
    for name in ('int2e_sph', 'int2e_ip1_sph'):
        out['c3_' + name + '_items'] = q3
        out['c3_' + name] = np.concatenate([o.ref.call(name, mol3, q)[1].ravel(order='F') for q in q3])
    # derivative family: (ij|nabla k l) on c0, (nabla i j|k) and (ij|nabla k) on the c2 molecule
    for name in ('int2e_ip2_sph', 'int2e_ip2_cart', 'int2e_ipip1_sph', 'int2e_ipip1_cart'):
        out['c0_' + name + '_items'] = qs[:40]
        out['c0_' + name] = np.concatenate([o.ref.call(name, mol0, q)[1].ravel(order='F') for q in qs[:40]])
    for name in ('int3c2e_ip1_sph', 'int3c2e_ip1_cart', 'int3c2e_ip2_sph', 'int3c2e_ip2_cart'):
        out['c2_' + name + '_items'] = tr
        out['c2_' + name] = np.concatenate([o.ref.call(name, mol2, t)[1].ravel(order='F') for t in tr])
    # long-range Coulomb
    m0 = mol0.copy()
    m0.env[8] = 0.3
    for name in ('int2e_sph', 'int2e_ip1_sph'):
        out['lr_c0_' + name + '_items'] = qs[:30]
        out['lr_c0_' + name] = np.concatenate([o.ref.call(name, m0, q)[1].ravel(order='F') for q in qs[:30]])
    m2 = mol2.copy()
    m2.env[8] = 0.5
    out['lr_c2_int3c2e_sph_items'] = tr[:40]
    out['lr_c2_int3c2e_sph'] = np.concatenate([o.ref.call('int3c2e_sph', m2, t)[1].ravel(order='F')
                                               for t in tr[:40]])
    out['lr_c2_int2c2e_sph_items'] = pr[:40]
    out['lr_c2_int2c2e_sph'] = np.concatenate([o.ref.call('int2c2e_sph', m2, t)[1].ravel(order='F')
                                               for t in pr[:40]])
    # short-range Coulomb erfc(omega r)/r (env[PTR_RANGE_OMEGA] < 0): the same items
    m0.env[8] = -0.3
    for name in ('int2e_sph', 'int2e_ip1_sph'):
        out['sr_c0_' + name + '_items'] = qs[:30]
        out['sr_c0_' + name] = np.concatenate([o.ref.call(name, m0, q)[1].ravel(order='F') for q in qs[:30]])
    m2.env[8] = -0.5
    out['sr_c2_int3c2e_sph_items'] = tr[:40]
    out['sr_c2_int3c2e_sph'] = np.concatenate([o.ref.call('int3c2e_sph', m2, t)[1].ravel(order='F')
                                               for t in tr[:40]])
    out['sr_c2_int2c2e_sph_items'] = pr[:40]
    out['sr_c2_int2c2e_sph'] = np.concatenate([o.ref.call('int2c2e_sph', m2, t)[1].ravel(order='F')
                                               for t in pr[:40]])
    # libcint's own errors per item against the long-double restatement (the referee): largest
    # absolute error, and largest relative error on elements above 1e-10 and above c of the
    # block's largest element (c = 1e-2 spherical, 1e-3 Cartesian), the bar a GPU test measures
    # itself against on ill-conditioned geometries
    for key, m in (('c4_int2e_sph', mol4), ('c4_int2e_cart', mol4), ('c4_int2e_ip1_sph', mol4),
                   ('c0_int2e_ip2_sph', mol0), ('c0_int2e_ip2_cart', mol0),
                   ('c0_int2e_ipip1_sph', mol0), ('c0_int2e_ipip1_cart', mol0),
                   ('c2_int3c2e_ip1_sph', mol2), ('c2_int3c2e_ip1_cart', mol2),
                   ('c2_int3c2e_ip2_sph', mol2), ('c2_int3c2e_ip2_cart', mol2)):
        name = key.split('_', 1)[1]
        rf, offs = o.referee(name, m, out[key + '_items'])
        ea, er = item_errors(out[key], rf, offs, 1e-2 if name.endswith('_sph') else 1e-3,
                             cart_scale(o, name, m, out[key + '_items']))
        out[key + '_liberr'] = ea
        out[key + '_librel'] = er
    kp = np.array([(i, k) for k in range(8) for i in range(8)], dtype=np.int32)
    out['kat_int2c2e_sph_items'] = kp
    out['kat_int2c2e_sph'] = np.concatenate([o.ref.call('int2c2e_sph', mol, t, nbas=nbas)[1]
                                             .ravel(order='F') for t in kp])
    # cache-size answers (out == NULL)
    f = o.ref.lib
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    cs = []
    for name, q in (('int2e_sph', (1, 3, 5, 7)), ('int2e_ip1_sph', (3, 1, 2, 0)),
                    ('int2e_cart', (1, 1, 0, 0)), ('int3c2e_sph', (2, 1, 3, 0)),
                    ('int2c2e_sph', (1, 3, 0, 0)), ('int2c2e_cart', (6, 2, 0, 0)),
                    ('int2c2e_sph', (5, 5, 0, 0))):
        shls = np.array(q, dtype=np.int32)
        r = getattr(f, name)(None, None, P(shls), P(mol.atm), mol.natm, P(mol.bas), nbas,
                             P(mol.env), None, None)
        cs.append((name, q, r))
    out['cache_names'] = np.array([c[0] for c in cs])
    out['cache_shls'] = np.array([c[1] for c in cs], dtype=np.int32)
    out['cache_sizes'] = np.array([c[2] for c in cs], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, 'ref_blocks.npz'), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == '__main__':
    main()
