"""Plan executions are a fixed sequence of stream-ordered operations (memsets, the integral kernels
on the caller's stream and a forked side stream, the output kernel), so they can be captured in a
CUDA graph and replayed.  A captured int2e_sph / int3c2e_sph execution replayed twice must give the
eager result bit for bit (every task owns its accumulator slot, the output kernel sums slots in a
fixed order); a captured J contraction (atomic adds) must agree to 1e-12."""
import numpy as np
import pytest

from libcint_gb300 import molecules as M

pytestmark = pytest.mark.gpu


def _eager_and_graph(cg, kind, mol, items):
    import torch
    plan = cg.Plan(kind, mol, items)
    eager = torch.zeros(plan.ncomp * plan.output_size, dtype=torch.float64, device='cuda')
    plan.execute(eager)
    torch.cuda.synchronize()
    out = torch.full_like(eager, np.nan)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.execute(out, s)            # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    out.fill_(np.nan)
    with torch.cuda.graph(g, stream=s):
        plan.execute(out, s)
    results = []
    for _ in range(2):
        out.fill_(np.nan)
        g.replay()
        torch.cuda.synchronize()
        results.append(out.clone())
    plan.close()
    return eager, results


@pytest.mark.parametrize('kind', ['INT2E_SPH', 'INT3C2E_SPH'])
def test_graph_replay_matches_eager(gpulib, kind):
    import torch
    mol = M.config0(seed=8)
    rng = np.random.RandomState(3)
    if kind == 'INT3C2E_SPH':
        items = np.stack([rng.randint(0, mol.nbas, 3000) for _ in range(3)], 1).astype(np.int32)
    else:
        qs = M.unique_quartets(mol.nbas)
        items = np.ascontiguousarray(qs[rng.choice(len(qs), 3000, replace=False)])
    eager, results = _eager_and_graph(gpulib, getattr(gpulib, kind), mol, items)
    for r in results:
        assert torch.equal(r, eager)


def test_graph_replay_j(gpulib):
    import torch
    from libcint_gb300.coulomb import CoulombPlans
    mol = M.config3(seed=2, natm=6, box=5.0)
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    rng = np.random.RandomState(0)
    d = rng.normal(0, 0.1, (nao, nao))
    dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    plans = CoulombPlans(mol)
    J_eager = plans.vj(dm)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plans.vj(dm, s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        J_graph = plans.vj(dm, s)
    g.replay()
    torch.cuda.synchronize()
    assert float((J_graph - J_eager).abs().max()) <= 1e-12
