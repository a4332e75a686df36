"""The allocation-free entry point cintgpu_int2e_sph_noalloc, through the C-ABI.

It exists for callers that cannot allocate device memory while they call us -- work enqueued in
a CUDA stream capture, or frameworks that own the device memory budget -- and keeps all of its
device scratch in one static 32 MiB device array.  This test compares two consecutive calls (two
different quartet batches, so the second call finds the first call's data in the shared array)
with the regular plan entry point on the same inputs, at the tolerance of the other parity tests.
It sits in its own file named to be collected last and passes alone in a fresh process as well.
"""
import ctypes
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests.test_gpu_parity import assert_block_close

pytestmark = pytest.mark.gpu


def _noalloc(gpulib):
    f = gpulib.lib().cintgpu_int2e_sph_noalloc
    vp = ctypes.c_void_p
    f.argtypes = [vp, vp, ctypes.c_int64, vp, ctypes.c_int, vp, ctypes.c_int, vp, vp]
    f.restype = ctypes.c_int
    return f


def test_noalloc_matches_plan_two_calls(gpulib):
    import torch
    f = _noalloc(gpulib)
    mol = M.config0(seed=21)
    qs_all = M.unique_quartets(mol.nbas)
    rng = np.random.RandomState(5)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for call in range(2):
        qs = np.ascontiguousarray(qs_all[rng.choice(len(qs_all), 400, replace=False)])
        plan = gpulib.Plan(gpulib.INT2E_SPH, mol, qs)
        ref = torch.zeros(plan.output_size, dtype=torch.float64, device='cuda')
        plan.execute(ref)
        out = torch.full((plan.output_size,), float('nan'), dtype=torch.float64, device='cuda')
        rc = f(ctypes.c_void_p(out.data_ptr()), P(qs), len(qs), P(mol.atm), mol.natm, P(mol.bas),
               mol.nbas, P(mol.env), None)
        assert rc == 0, gpulib.last_error()
        torch.cuda.synchronize()
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all()
        off = 0
        for q in qs:
            nb = int(np.prod([mol.nsph(s) for s in q]))
            assert_block_close(got[off:off + nb], want[off:off + nb], 'noalloc call %d %s' % (call, q))
            off += nb
        plan.close()


def test_noalloc_rejects_oversized_batch(gpulib):
    import torch
    f = _noalloc(gpulib)
    mol = M.config1(seed=0)
    qs = np.ascontiguousarray(np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_quartets.npz'))['quartets'][:60000])
    out = torch.zeros(8, dtype=torch.float64, device='cuda')
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = f(ctypes.c_void_p(out.data_ptr()), P(qs), len(qs), P(mol.atm), mol.natm, P(mol.bas),
           mol.nbas, P(mol.env), None)
    assert rc == -4 and 'limited to' in gpulib.last_error()
