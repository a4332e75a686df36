"""h and i shells (l = 5, 6), the top of the drop-in's range: the contraction-first kernel takes its
member-at-a-time stage 3 (lj or ll above 3), 12-13 Rys roots, the 48 KB shared-memory group and the
separate output transform (the fused one would need gigabytes of per-warp scratch for such
blocks).  Blocks are compared with the oracle element by element through both the drop-in and a
batched plan, for int2e (sph, cart) and int3c2e (sph)."""
import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests.test_gpu_parity import assert_block_close, cart_scale

pytestmark = pytest.mark.gpu


def high_l_basis():
    """3 atoms; shells (l, exponents, contraction columns): i with 2 primitives, h with 1
    primitive x 2 columns, g, d, s."""
    natm = 3
    env = np.zeros(4000)
    atm = np.zeros((natm, M.ATM_SLOTS), np.int32)
    off = M.PTR_ENV_START
    xyz = [(0.0, 0.0, 0.0), (0.9, -0.4, 0.7), (-0.6, 1.1, 0.3)]
    for i in range(natm):
        atm[i, M.CHARGE_OF] = 2
        atm[i, M.PTR_COORD] = off
        env[off:off + 3] = xyz[i]
        off += 3
    spec = [(0, 6, [1.6, 0.7], [[0.6, 0.5]]), (1, 5, [1.1], [[1.0], [0.4]]), (2, 4, [0.9], [[1.0]]),
            (0, 2, [1.3], [[1.0]]), (1, 0, [2.0], [[1.0]])]
    bas = []
    for at, l, ex, cols in spec:
        pe = off
        env[off:off + len(ex)] = ex
        off += len(ex)
        pc = off
        for col in cols:
            for p, e in enumerate(ex):
                env[off] = col[p] * M.gto_norm(l, e)
                off += 1
        bas.append([at, l, len(ex), len(cols), 0, pe, pc, 0])
    return M.Mol(atm, np.array(bas, np.int32), env, 'high_l')


QUARTETS = [(0, 0, 0, 0), (0, 1, 0, 1), (1, 1, 2, 3), (0, 4, 0, 3), (0, 0, 4, 4), (2, 1, 0, 3),
            (1, 0, 1, 2)]
TRIPLES = [(0, 0, 2), (1, 0, 0), (3, 4, 0), (1, 1, 1)]


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_cart'])
def test_high_l_dropin_and_plan(gpulib, oracle, name):
    import torch
    mol = high_l_basis()
    sph = name.endswith('_sph')
    qs = np.array(QUARTETS, dtype=np.int32)
    plan = gpulib.Plan(gpulib.INT2E_SPH if sph else gpulib.INT2E_CART, mol, qs)
    out = torch.zeros(plan.output_size, dtype=torch.float64, device='cuda')
    plan.execute(out)
    res = out.cpu().numpy()
    plan.close()
    off = 0
    for q in QUARTETS:
        _, ref = oracle.port.call(name, mol, q)
        scale = cart_scale(oracle, name, mol, q)
        _, got = gpulib.dropin(name, mol, q)
        assert_block_close(got, ref, '%s drop-in %s' % (name, q), scale)
        nb = ref.size
        assert_block_close(res[off:off + nb], ref.ravel(order='F'), '%s plan %s' % (name, q), scale)
        off += nb


def test_high_l_3c2e(gpulib, oracle):
    mol = high_l_basis()
    for t in TRIPLES:
        _, ref = oracle.port.call('int3c2e_sph', mol, t)
        _, got = gpulib.dropin('int3c2e_sph', mol, t)
        assert_block_close(got, ref, '3c2e %s' % (t,), cart_scale(oracle, 'int3c2e_sph', mol, t))


def _plan_blocks(gpulib, mol, items, env=None):
    import os
    import torch
    old = {k: os.environ.get(k) for k in (env or {})}
    os.environ.update(env or {})
    try:
        plan = gpulib.Plan(gpulib.INT2E_SPH, mol, items)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    out = torch.zeros(plan.output_size, dtype=torch.float64, device='cuda')
    plan.execute(out)
    res = out.cpu().numpy()
    plan.close()
    return res


def test_c1_ff_classes(gpulib, oracle):
    """Benchmark quartets whose transfer side holds an f shell (kernel-order lj or ll = 3, the
    largest transfers the contraction-first kernel takes by default), against the oracle.
    Default plans: the 1e-12 absolute bar, and 1e-8 relative on uncancelled elements (the transfer
    after contraction multiplies the three axes' rounding amplifications; measured up to 1.4e-9 on
    these quartets, i.e. ~1e-13 of the block scale).  With CINTGPU_PER_PRIMITIVE_L=3 these classes
    transfer per primitive like libcint (at about half the c1 throughput) and meet the strict
    relative gate as well."""
    import os
    mol = M.config1(seed=0)
    qs = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_quartets.npz'))['quartets']
    L = mol.bas[:, M.ANG_OF]
    lmin_bra = np.minimum(L[qs[:, 0]], L[qs[:, 1]])
    lmin_ket = np.minimum(L[qs[:, 2]], L[qs[:, 3]])
    sel = qs[(lmin_bra == 3) | (lmin_ket == 3)][:120]
    assert len(sel) >= 60
    refs = [oracle.port.call('int2e_sph', mol, q)[1] for q in sel]
    scales = [cart_scale(oracle, 'int2e_sph', mol, q) for q in sel]
    for env, rel in ((None, 1e-8), ({'CINTGPU_PER_PRIMITIVE_L': '3'}, None)):
        res = _plan_blocks(gpulib, mol, sel, env)
        off = 0
        for q, ref, sc in zip(sel, refs, scales):
            nb = ref.size
            got = res[off:off + nb]
            if rel is None:
                assert_block_close(got, ref.ravel(order='F'), 'c1 per-primitive %s' % (q,), sc)
            else:
                d = np.abs(got - ref.ravel(order='F'))
                assert d.max() <= 1e-12, 'c1 %s max abs diff %.3e' % (q, d.max())
                big = (np.abs(ref.ravel(order='F')) > 1e-3 * sc) & (np.abs(ref.ravel(order='F')) > 1e-10)
                if big.any():
                    r = (d[big] / np.abs(ref.ravel(order='F')[big])).max()
                    assert r <= rel, 'c1 %s max rel diff %.3e' % (q, r)
            off += nb
