"""CINTOpt with content: int2e_optimizer registers a side table (the shell pairs' primitive data,
built on first use and shared between threads) that the drop-in calls made with it reuse; calls
with and without the optimizer, from several threads at once, give identical blocks, and
CINTdel_optimizer releases it."""
import ctypes
import threading

import numpy as np
import pytest

from libcint_gb300 import molecules as M

pytestmark = pytest.mark.gpu


def _call(L, name, mol, q, opt):
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    n = int(np.prod([mol.nsph(int(s)) for s in q])) * (3 if '_ip1' in name else 1)
    out = np.zeros(n)
    shls = np.ascontiguousarray(q, dtype=np.int32)
    flag = getattr(L, name)(P(out), None, P(shls), P(mol.atm), mol.natm, P(mol.bas), mol.nbas,
                            P(mol.env), opt, None)
    return flag, out


@pytest.mark.parametrize('name,optname', [('int2e_sph', 'int2e_optimizer'),
                                          ('int2e_ip1_sph', 'int2e_ip1_optimizer')])
def test_optimizer_threads(gpulib, name, optname):
    L = gpulib.lib()
    mol = M.config0(seed=4)
    qs = M.unique_quartets(mol.nbas)
    qs = qs[np.random.RandomState(1).choice(len(qs), 240, replace=False)]
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    opt = ctypes.c_void_p()
    getattr(L, optname)(ctypes.byref(opt), P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env))
    assert opt.value
    ref = [_call(L, name, mol, q, None) for q in qs]
    got = [None] * len(qs)

    def worker(k):
        for t in range(k, len(qs), 6):
            got[t] = _call(L, name, mol, qs[t], opt)
    th = [threading.Thread(target=worker, args=(k,)) for k in range(6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for (f0, a), (f1, b) in zip(ref, got):
        assert f0 == f1
        np.testing.assert_array_equal(a, b)
    # a second pass reuses the cached pairs
    again = [_call(L, name, mol, q, opt) for q in qs[:40]]
    for (f0, a), (f1, b) in zip(ref[:40], again):
        assert f0 == f1
        np.testing.assert_array_equal(a, b)
    L.CINTdel_optimizer(ctypes.byref(opt))
    assert not opt.value
