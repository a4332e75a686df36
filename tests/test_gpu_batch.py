"""The one-shot host-buffer entry cintgpu_batch_host, through the C-ABI.  Without offsets it cuts
the item list into chunks (512 items, growing to 12288) planned on host threads while the GPU runs
earlier chunks; its output must equal one device plan over the whole list (same layout:
component-major, blocks back to back) to the tolerance of the other parity tests, and the oracle
on a sample."""
import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests.test_gpu_parity import assert_block_close

pytestmark = pytest.mark.gpu


def _plan_out(cg, kind, mol, items, offsets=None):
    import torch
    p = cg.Plan(kind, mol, items, offsets)
    out = torch.zeros(p.ncomp * p.output_size, dtype=torch.float64, device='cuda')
    p.execute(out)
    torch.cuda.synchronize()
    r = out.cpu().numpy().reshape(p.ncomp, p.output_size)
    p.close()
    return r


@pytest.mark.parametrize('kind,n', [('INT2E_SPH', 10000), ('INT2E_CART', 4097), ('INT2E_IP1_SPH', 9000),
                                    ('INT3C2E_SPH', 9000)])
def test_batch_host_chunks_match_plan(gpulib, oracle, kind, n):
    cg = gpulib
    k = getattr(cg, kind)
    mol = M.config0(seed=4)
    rng = np.random.RandomState(n)
    if kind.startswith('INT3C2E'):
        items = np.stack([rng.randint(0, mol.nbas, n) for _ in range(3)], 1).astype(np.int32)
    else:
        qs = M.unique_quartets(mol.nbas)
        items = np.ascontiguousarray(qs[rng.choice(len(qs), n, replace=False)])
    got = cg.batch_host(k, mol, items)
    want = _plan_out(cg, k, mol, items)
    assert got.shape == want.shape
    assert_block_close(got, want, 'batch_host %s' % kind)
    # a few items against the oracle, across the chunk boundaries
    name = kind.lower()
    sph = name.endswith('_sph')
    nsh = items.shape[1]
    sizes = np.array([np.prod([mol.nsph(s) if sph else mol.ncart(s) for s in it]) for it in items])
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    ncomp = got.shape[0]
    for q in sorted({0, 511, 512, 1151, 1152, 4095, 4096, n - 1} & set(range(n))):
        _, ref = oracle.port.call(name, mol, items[q][:nsh])
        for c in range(ncomp):
            r = ref[..., c] if ncomp > 1 else ref
            assert_block_close(got[c, offs[q]:offs[q] + sizes[q]], r.ravel(order='F'),
                               'batch_host %s item %d comp %d' % (kind, q, c))


def test_batch_host_offsets_and_rejects_j(gpulib):
    cg = gpulib
    mol = M.config0(seed=5)
    qs = M.unique_quartets(mol.nbas)[:300].astype(np.int32)
    sizes = np.array([np.prod([mol.nsph(s) for s in q]) for q in qs])
    offsets = np.zeros(len(qs), np.int64)   # reversed order with gaps
    pos = 3
    for q in range(len(qs) - 1, -1, -1):
        offsets[q] = pos
        pos += sizes[q] + 2
    got = cg.batch_host(cg.INT2E_SPH, mol, qs, offsets)
    want = _plan_out(cg, cg.INT2E_SPH, mol, qs, offsets)
    assert_block_close(got, want, 'batch_host offsets')
    with pytest.raises(cg.CintGpuError):
        cg.batch_host(7, mol, qs)


@pytest.mark.parametrize('kind,n', [('INT2E_SPH', 6000), ('INT3C2E_SPH', 30000), ('INT2C2E_CART', 3000)])
def test_batch_device_matches_plan(gpulib, kind, n):
    """cintgpu_batch_device (the host-buffer pipeline writing into a device buffer) gives one
    device plan's output; a two-component kind is refused"""
    import torch
    cg = gpulib
    k = getattr(cg, kind)
    mol = M.config0(seed=6)
    rng = np.random.RandomState(n)
    nsh = {'INT2E_SPH': 4, 'INT3C2E_SPH': 3, 'INT2C2E_CART': 2}[kind]
    if nsh == 4:
        qs = M.unique_quartets(mol.nbas)
        items = np.ascontiguousarray(qs[rng.choice(len(qs), n, replace=False)])
    else:
        items = np.stack([rng.randint(0, mol.nbas, n) for _ in range(nsh)], 1).astype(np.int32)
    want = _plan_out(cg, k, mol, items)[0]
    out = torch.full((want.size + 7,), 7.0, dtype=torch.float64, device='cuda')
    cg.batch_device(k, mol, items, out)
    got = out.cpu().numpy()
    assert (got[want.size:] == 7.0).all()                  # nothing written past the blocks
    assert_block_close(got[:want.size], want, 'batch_device %s' % kind)
    with pytest.raises(cg.CintGpuError):
        cg.batch_device(cg.INT2E_IP1_SPH, mol, items[:10] if nsh == 4 else M.unique_quartets(mol.nbas)[:10], out)
