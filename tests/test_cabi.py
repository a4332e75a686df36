"""The C-ABI library: loads without a GPU, exports every function include/cintgpu.h declares, its
host-only parts agree with libcint (cart->sph rows, basis helpers, cache-size answers), and the
compute entry points fail loudly when no GPU is usable (no CPU fallback).  CPU only."""
import ctypes
import os
import re

import numpy as np
import pytest

from libcint_gb300 import molecules as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(ROOT, 'include', 'cintgpu.h')).read()
    src = re.sub(r'/\*.*?\*/', ' ', src, flags=re.S)
    src = '\n'.join(l for l in src.splitlines() if not l.strip().startswith('#'))
    names = []
    for chunk in ' '.join(src.split()).split(';'):
        chunk = chunk.strip()
        if not chunk or chunk.startswith('typedef') or '{' in chunk or '}' in chunk:
            continue
        m = re.search(r'(\w+)\s*\(', chunk)
        if m:
            names.append(m.group(1))
    return names


def test_library_exports_every_declared_function(gpulib):
    L = gpulib.lib()
    names = _declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_cart2sph_rows_match_oracle(gpulib, oracle):
    L = gpulib.lib()
    ol = oracle.port.lib
    for l in range(0, 7):
        nc = (l + 1) * (l + 2) // 2
        ns = 2 * l + 1 if l > 1 else nc
        a = np.zeros(ns * nc)
        b = np.zeros(ns * nc)
        assert L.cintgpu_cart2sph(l, a.ctypes.data_as(ctypes.c_void_p)) == ns
        ol.oracle_cart2sph_coeff(l, b.ctypes.data_as(ctypes.c_void_p))
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-15)


def test_basis_helpers(gpulib):
    L = gpulib.lib()
    for l in range(6):
        for a in (0.05, 1.0, 37.5):
            assert abs(L.CINTgto_norm(l, a) - M.gto_norm(l, a)) <= 1e-14 * M.gto_norm(l, a)
    mol = M.config0(seed=1)
    L.CINTtot_cgto_spheric.restype = ctypes.c_int
    assert L.CINTtot_cgto_spheric(mol.bas.ctypes.data_as(ctypes.c_void_p), mol.nbas) == 104
    loc = np.zeros(mol.nbas, dtype=np.int32)
    L.CINTshells_spheric_offset(loc.ctypes.data_as(ctypes.c_void_p),
                                mol.bas.ctypes.data_as(ctypes.c_void_p), mol.nbas)
    np.testing.assert_array_equal(loc, mol.ao_loc()[:-1])


def test_cache_size_query_matches_libcint(gpulib):
    """out == NULL returns libcint's cache size (src/cint2e.c:801-816); pure host path."""
    fx = np.load(os.path.join(ROOT, 'tests', 'golden', 'ref_blocks.npz'))
    mol, nbas = M.kat_basis()
    L = gpulib.lib()
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for name, shls, want in zip(fx['cache_names'], fx['cache_shls'], fx['cache_sizes']):
        s = np.ascontiguousarray(shls, dtype=np.int32)
        got = getattr(L, str(name))(None, None, P(s), P(mol.atm), mol.natm, P(mol.bas), nbas,
                                    P(mol.env), None, None)
        assert got == want, (name, got, want)


def test_no_gpu_fails_loudly(gpulib):
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    mol = M.config0(seed=0)
    with pytest.raises(gpulib.CintGpuError, match='CUDA'):
        gpulib.Plan(gpulib.INT2E_SPH, mol, M.unique_quartets(mol.nbas)[:4])
    L = gpulib.lib()
    before = L.cintgpu_dropin_failures()
    flag, blk = gpulib.dropin('int2e_sph', mol, (1, 0, 0, 0))
    # a failed call returns 0 like a screened block, but its block is NaN (a screened block is
    # zeros), it is counted and it leaves a message
    assert flag == 0 and np.isnan(blk).all() and gpulib.last_error()
    assert L.cintgpu_dropin_failures() == before + 1
    # the CINT2 form and a strided dims layout: only the block's own elements are NaN
    out = np.zeros(7 * 7 * 7 * 7)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    shls = np.array([2, 1, 0, 0], np.int32)
    dims = np.array([7, 7, 7, 7], np.int32)
    assert L.int2e_sph(P(out), P(dims), P(shls), P(mol.atm), mol.natm, P(mol.bas), mol.nbas,
                       P(mol.env), None, None) == 0
    blockview = out.reshape(7, 7, 7, 7, order='F')
    n = [mol.nsph(int(x)) for x in shls]
    assert np.isnan(blockview[:n[0], :n[1], :n[2], :n[3]]).all()
    assert np.isnan(out).sum() == np.prod(n)
    assert L.cintgpu_dropin_failures() == before + 2


@pytest.mark.parametrize('name,nsh', [('int2e_sph', 4), ('int2e_cart', 4), ('int2e_ip1_sph', 4),
                                      ('int2e_ip1_cart', 4), ('int3c2e_sph', 3),
                                      ('int3c2e_cart', 3), ('int2c2e_sph', 2), ('int2c2e_cart', 2),
                                      ('int2e_ip2_sph', 4), ('int2e_ip2_cart', 4),
                                      ('int3c2e_ip1_sph', 3), ('int3c2e_ip1_cart', 3),
                                      ('int3c2e_ip2_sph', 3), ('int3c2e_ip2_cart', 3)])
def test_cache_size_query_matches_libcint_live(gpulib, oracle, name, nsh):
    """out == NULL answers for 200 random shell sets of the KAT basis (general contractions,
    l <= 4) and of c2 (1-6 primitives, auxiliary l <= 4), against libcint compiled from its
    sources; a pure host path."""
    if oracle.ref is None:
        pytest.skip('libcint not built from sources on this machine')
    L = gpulib.lib()
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    kat, nk = M.kat_basis()
    c2, _ = M.config2(seed=1, natm=4, box=4.0)
    rng = np.random.RandomState(nsh)
    for mol, nb, top in ((kat, nk, 8), (c2, c2.nbas, c2.nbas)):
        for _ in range(100):
            s = np.ascontiguousarray(rng.randint(0, top, 4), dtype=np.int32)
            got = getattr(L, name)(None, None, P(s), P(mol.atm), mol.natm, P(mol.bas), nb,
                                   P(mol.env), None, None)
            want = getattr(oracle.ref.lib, name)(None, None, P(s), P(mol.atm), mol.natm,
                                                 P(mol.bas), nb, P(mol.env), None, None)
            assert got == want, (name, s[:nsh].tolist(), got, want)


def test_new_entries_reject_bad_arguments_before_the_device(gpulib):
    """argument checks of the device-output batch and the density-fitting handle run before any
    device work, so they answer the same with or without a GPU: a two-component kind, a J kind,
    pair descriptors outside the AO range or above the AO-pair limit"""
    L = gpulib.lib()
    mol = M.config0(seed=0)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    q = np.ascontiguousarray(M.unique_quartets(mol.nbas)[:4], dtype=np.int32)
    out = ctypes.c_void_p(16)   # never dereferenced: the checks fail first
    for kind in (gpulib.INT2E_IP1_SPH, 7):      # a two-component kind; J_BUILD
        rc = L.cintgpu_batch_device(kind, out, P(q), len(q), P(mol.atm), mol.natm, P(mol.bas),
                                    mol.nbas, P(mol.env))
        assert rc == -1 and gpulib.last_error()
    h = ctypes.c_void_p()
    for desc, nao in (([0, 0, 3, 3], 2), ([-1, 0, 1, 1], 4), ([0, 0, 80, 80], 200)):
        d = np.array(desc, np.int32)
        assert L.cintgpu_df_create(ctypes.byref(h), P(d), 1, nao, 10) == -1
        assert 'df: pair 0' in gpulib.last_error() and not h.value
    assert L.cintgpu_df_create(ctypes.byref(h), None, 1, 4, 10) == -1
    assert L.cintgpu_df_create(ctypes.byref(h), None, 0, 0, 10) == -1
