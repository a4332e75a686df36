"""Coulomb-like (J) and exchange (K) contractions and the adjoint on the GPU, checked against the
oracle's ERIs and int2e_ip1 (contracted on the host), against int2e_ip1 formed on the GPU, and
against central finite differences (h = 1e-4 Bohr for coordinates, relative 1e-5 for exponents).

Tolerances: J, K and the gradients agree with the integral-level references to 1e-10 relative to
their largest element (the adjoint's target); finite differences to 1e-7 (their truncation error
is ~h^2 |d3L|)."""
import numpy as np
import pytest

from libcint_gb300 import molecules as M

pytestmark = pytest.mark.gpu


def _system(natm=3, seed=11):
    mol = M.config3(seed=seed, natm=natm, box=3.5)
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    rng = np.random.RandomState(seed)
    d = rng.normal(0, 0.1, (nao, nao))
    return mol, 0.5 * (d + d.T)


def _oracle_j_energy(oracle, mol, dm):
    loc = mol.ao_loc()
    J = np.zeros_like(dm)
    for (i, j, k, l) in M.unique_quartets(mol.nbas):
        _, blk = oracle.port.call('int2e_sph', mol, (i, j, k, l))
        # every distinct permutation of the unique quartet contributes
        seen = set()
        for (a, b, c, d, t) in ((i, j, k, l, 'ijkl'), (j, i, k, l, 'jikl'), (i, j, l, k, 'ijlk'),
                                (j, i, l, k, 'jilk'), (k, l, i, j, 'klij'), (l, k, i, j, 'lkij'),
                                (k, l, j, i, 'klji'), (l, k, j, i, 'lkji')):
            if (a, b, c, d) in seen:
                continue
            seen.add((a, b, c, d))
            g = np.transpose(blk, ['ijkl'.index(ch) for ch in t])
            J[loc[a]:loc[a + 1], loc[b]:loc[b + 1]] += np.einsum(
                'abcd,cd->ab', g, dm[loc[c]:loc[c + 1], loc[d]:loc[d + 1]])
    return J, 0.5 * (dm * J).sum()


def test_j_and_energy_match_oracle(gpulib, oracle):
    import torch
    from libcint_gb300.coulomb import CoulombPlans
    mol, dm = _system()
    Jref, Eref = _oracle_j_energy(oracle, mol, dm)
    plans = CoulombPlans(mol)
    E, J = plans.energy(torch.as_tensor(dm, device='cuda'))
    J = J.cpu().numpy()
    assert np.abs(J - Jref).max() <= 1e-10 * np.abs(Jref).max()
    assert abs(float(E) - Eref) <= 1e-10 * abs(Eref)


@pytest.mark.parametrize('basis', ['c3', 'two_column'])
def test_k_and_jk_match_oracle(gpulib, oracle, basis):
    """K = einsum('ijkl,jl->ik') of the oracle's full ERI tensor, from a K_BUILD plan and from a
    JK_BUILD plan (whose J must equal the J_BUILD plan's); the two_column basis has d shells with
    two contraction columns (shell-level coincidences across columns)."""
    import torch
    from libcint_gb300.coulomb import CoulombPlans
    from tests.test_jk_algebra import _basis, _eri_full
    if basis == 'c3':
        mol, _ = _system()
    else:
        mol = _basis()
    eri, _ = _eri_full(oracle, mol)
    n = eri.shape[0]
    rng = np.random.RandomState(4)
    d = rng.normal(0, 0.1, (n, n))
    dm = 0.5 * (d + d.T)
    Jref = np.einsum('ijkl,kl->ij', eri, dm)
    Kref = np.einsum('ijkl,jl->ik', eri, dm)
    plans = CoulombPlans(mol)
    dmt = torch.as_tensor(dm, device='cuda')
    K = plans.vk(dmt).cpu().numpy()
    J2, K2 = (x.cpu().numpy() for x in plans.get_jk(dmt))
    J = plans.vj(dmt).cpu().numpy()
    tol = 1e-10
    assert np.abs(K - Kref).max() <= tol * np.abs(Kref).max(), np.abs(K - Kref).max()
    assert np.abs(K2 - Kref).max() <= tol * np.abs(Kref).max(), np.abs(K2 - Kref).max()
    assert np.abs(J2 - Jref).max() <= tol * np.abs(Jref).max(), np.abs(J2 - Jref).max()
    assert np.abs(J2 - J).max() <= 1e-13 * np.abs(Jref).max()
    assert np.abs(K - K.T).max() <= 1e-14 * np.abs(Kref).max()


def _oracle_grad_ip1(oracle, mol, dm):
    """dL/dR = -1/2 sum_q w_q sum D D (nabla ...) over the four centres, libcint-style ip1."""
    loc = mol.ao_loc()
    atom = mol.bas[:, M.ATOM_OF]
    grad = np.zeros((mol.natm, 3))
    for q in M.unique_quartets(mol.nbas):
        i, j, k, l = (int(v) for v in q)
        w = (2.0 if i != j else 1.0) * (2.0 if k != l else 1.0) * (2.0 if (i, j) != (k, l) else 1.0)
        vs = []
        for perm in ((i, j, k, l), (j, i, k, l), (k, l, i, j)):
            _, blk = oracle.port.call('int2e_ip1_sph', mol, perm)
            a, b, c, d = perm
            v = np.einsum('ijklx,ij,kl->x', blk, dm[loc[a]:loc[a + 1], loc[b]:loc[b + 1]],
                          dm[loc[c]:loc[c + 1], loc[d]:loc[d + 1]]) * (-0.5 * w)
            vs.append(v)
            grad[atom[perm[0]]] += v
        grad[atom[l]] -= vs[0] + vs[1] + vs[2]
    return grad


def test_adjoint_matches_oracle_ip1_and_gpu_ip1(gpulib, oracle):
    import torch
    from libcint_gb300.coulomb import CoulombPlans, grad_via_ip1
    mol, dm = _system()
    gref = _oracle_grad_ip1(oracle, mol, dm)
    plans = CoulombPlans(mol)
    dmt = torch.as_tensor(dm, device='cuda')
    g, _ = plans.grad(dmt)
    g = g.cpu().numpy()
    scale = np.abs(gref).max()
    assert np.abs(g - gref).max() <= 1e-10 * scale, np.abs(g - gref).max()
    gi = grad_via_ip1(mol, dmt).cpu().numpy()
    assert np.abs(gi - gref).max() <= 1e-10 * scale
    # translational invariance of the total
    assert np.abs(g.sum(0)).max() <= 1e-10 * scale


def test_adjoint_matches_finite_differences(gpulib):
    import torch
    from libcint_gb300.coulomb import CoulombPlans, atom_coords, with_geometry
    mol, dm = _system()
    dmt = torch.as_tensor(dm, device='cuda')
    g, ga = CoulombPlans(mol, with_exponents=True).grad(dmt)
    g = g.cpu().numpy()
    ga = ga.cpu().numpy()
    R = atom_coords(mol)
    h = 1e-4
    for a in range(mol.natm):
        for x in range(3):
            Rp, Rm = R.copy(), R.copy()
            Rp[a, x] += h
            Rm[a, x] -= h
            Ep = float(CoulombPlans(with_geometry(mol, Rp)).energy(dmt)[0])
            Em = float(CoulombPlans(with_geometry(mol, Rm)).energy(dmt)[0])
            assert abs((Ep - Em) / (2 * h) - g[a, x]) <= 1e-7 * max(1.0, abs(g[a, x])), (a, x)
    from libcint_gb300.coulomb import exponents_of
    ex = exponents_of(mol)
    for p in range(0, len(ex), max(1, len(ex) // 7)):
        hp = 1e-5 * ex[p]
        ep, em = ex.copy(), ex.copy()
        ep[p] += hp
        em[p] -= hp
        Ep = float(CoulombPlans(with_geometry(mol, exps=ep)).energy(dmt)[0])
        Em = float(CoulombPlans(with_geometry(mol, exps=em)).energy(dmt)[0])
        fd = (Ep - Em) / (2 * hp)
        assert abs(fd - ga[p]) <= 1e-7 * max(1.0, abs(ga[p])), (p, fd, ga[p])


def test_autograd_function(gpulib):
    import torch
    from libcint_gb300.coulomb import CoulombPlans, atom_coords, coulomb_energy, exponents_of
    mol, dm = _system()
    coords = torch.tensor(atom_coords(mol), dtype=torch.float64, requires_grad=True)
    exps = torch.tensor(exponents_of(mol), dtype=torch.float64, requires_grad=True)
    dmt = torch.tensor(dm, dtype=torch.float64, device='cuda', requires_grad=True)
    E = coulomb_energy(coords, exps, dmt, mol)
    E.backward()
    g, ga = CoulombPlans(mol, with_exponents=True).grad(dmt.detach())
    np.testing.assert_allclose(coords.grad.cpu().numpy(), g.cpu().numpy(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(exps.grad.cpu().numpy(), ga.cpu().numpy(), rtol=0, atol=1e-12)
    _, J = CoulombPlans(mol).energy(dmt.detach())
    np.testing.assert_allclose(dmt.grad.cpu().numpy(), J.cpu().numpy(), rtol=0, atol=1e-12)


def test_j_high_l_per_primitive_classes(gpulib, oracle):
    """J over every unique quartet of a basis with g, h and i shells: classes with lj or ll >= 4
    take the per-primitive kernel (third task group, its own J scratch slots), the rest the
    contraction-first one; both against the oracle's ERIs contracted on the host."""
    import torch
    from libcint_gb300.coulomb import CoulombPlans
    from tests.test_gpu_high_l import high_l_basis
    mol = high_l_basis()
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    rng = np.random.RandomState(2)
    d = rng.normal(0, 0.1, (nao, nao))
    dm = 0.5 * (d + d.T)
    Jref, Eref = _oracle_j_energy(oracle, mol, dm)
    plans = CoulombPlans(mol)
    E, J = plans.energy(torch.as_tensor(dm, device='cuda'))
    J = J.cpu().numpy()
    assert np.abs(J - Jref).max() <= 1e-10 * np.abs(Jref).max()
    assert abs(float(E) - Eref) <= 1e-10 * abs(Eref)


def _grad_with(mol, dmt, adjoint, quartets=None, exponents=False):
    import os
    from libcint_gb300.coulomb import CoulombPlans
    old = os.environ.get('CINTGPU_ADJOINT')
    os.environ['CINTGPU_ADJOINT'] = adjoint
    try:
        # the adjoint plan is built by the first grad call
        g, ga = CoulombPlans(mol, quartets, with_exponents=exponents).grad(dmt)
        return (g.cpu().numpy(), ga.cpu().numpy()) if exponents else g.cpu().numpy()
    finally:
        if old is None:
            os.environ.pop('CINTGPU_ADJOINT')
        else:
            os.environ['CINTGPU_ADJOINT'] = old


@pytest.mark.parametrize('case', ['c3', 'g_shells', 'long_range', 'short_range'])
def test_contraction_first_adjoint_matches_per_component(gpulib, case):
    """The two adjoint kernels: contraction first (densities carried through the transfers, the
    default) and per Cartesian component (CINTGPU_ADJOINT=component) on every unique quartet of a
    c3-type system, of a basis with s..g shells (1-3 primitives; without the (gg|gg) quartets,
    whose raised g arrays exceed the per-component kernel), and with the long-range operator;
    agreement to 1e-11 of the largest gradient element."""
    import torch
    quartets = None
    if case == 'g_shells':
        b = M._Builder()
        rng = np.random.RandomState(4)
        for a in range(3):
            at = b.atom(1 + a, tuple(rng.uniform(-1.2, 1.2, 3)))
            for l, npr in ((0, 2), (1, 3), (2, 2), (3, 1), (4, 2)):
                ex = sorted(rng.uniform(0.3, 4.0, npr), reverse=True)
                b.shell(at, l, ex, [M.gto_norm(l, e) * rng.uniform(0.3, 1.0) for e in ex])
        mol = b.mol('g shells')
        q = np.asarray(M.unique_quartets(mol.nbas))
        quartets = q[(mol.bas[q, M.ANG_OF] < 4).any(axis=1)]
        nao = sum(mol.nsph(i) for i in range(mol.nbas))
        d = rng.normal(0, 0.1, (nao, nao))
        dm = 0.5 * (d + d.T)
    else:
        mol, dm = _system(natm=5, seed=3)
        if case == 'long_range':
            mol.env[8] = 0.6           # env[PTR_RANGE_OMEGA]: long-range Coulomb
        elif case == 'short_range':
            mol.env[8] = -0.6
    dmt = torch.as_tensor(dm, device='cuda')
    g1 = _grad_with(mol, dmt, 'contraction', quartets)
    g2 = _grad_with(mol, dmt, 'component', quartets)
    scale = np.abs(g2).max()
    assert scale > 0
    assert np.abs(g1 - g2).max() <= 1e-11 * scale, np.abs(g1 - g2).max() / scale
    if case == 'g_shells':
        # every quartet, (gg|gg) included, against int2e_ip1 formed on the GPU and contracted
        from libcint_gb300.coulomb import grad_via_ip1
        ga = _grad_with(mol, dmt, 'contraction')
        gi = grad_via_ip1(mol, dmt).cpu().numpy()
        assert np.abs(ga - gi).max() <= 1e-10 * np.abs(gi).max(), np.abs(ga - gi).max() / np.abs(gi).max()


def test_contraction_first_exponent_adjoint_matches_per_component(gpulib):
    """Coordinate and primitive-exponent gradients from the contraction-first exponent adjoint
    against the per-component kernel on a c3-type system and on s..f shells with up to 3
    primitives: 1e-11 of each gradient's largest element."""
    import torch
    mol, dm = _system(natm=4, seed=5)
    dmt = torch.as_tensor(dm, device='cuda')
    g1, a1 = _grad_with(mol, dmt, 'contraction', exponents=True)
    g2, a2 = _grad_with(mol, dmt, 'component', exponents=True)
    assert np.abs(g1 - g2).max() <= 1e-11 * np.abs(g2).max()
    assert np.abs(a1 - a2).max() <= 1e-11 * np.abs(a2).max()
    b = M._Builder()
    rng = np.random.RandomState(8)
    for a in range(2):
        at = b.atom(1 + a, tuple(rng.uniform(-1.0, 1.0, 3)))
        for l, npr in ((0, 3), (1, 2), (2, 2), (3, 2)):
            ex = sorted(rng.uniform(0.3, 4.0, npr), reverse=True)
            b.shell(at, l, ex, [M.gto_norm(l, e) * rng.uniform(0.3, 1.0) for e in ex])
    mol = b.mol('s..f')
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    d = rng.normal(0, 0.1, (nao, nao))
    dmt = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    # the per-component exponent kernel cannot hold (ff|ff) and (ff|fd): compare without them
    q = np.asarray(M.unique_quartets(mol.nbas))
    part = q[(mol.bas[q, M.ANG_OF] == 3).sum(axis=1) < 3]
    g1, a1 = _grad_with(mol, dmt, 'contraction', part, exponents=True)
    g2, a2 = _grad_with(mol, dmt, 'component', part, exponents=True)
    assert np.abs(g1 - g2).max() <= 1e-11 * np.abs(g2).max()
    assert np.abs(a1 - a2).max() <= 1e-11 * np.abs(a2).max()
    # every quartet: coordinates against the coordinate-only kernel, exponents of the f shells
    # against central differences of the energy (relative step 1e-5)
    from libcint_gb300.coulomb import CoulombPlans, exponents_of, with_geometry
    g, ga = _grad_with(mol, dmt, 'contraction', exponents=True)
    gc = _grad_with(mol, dmt, 'contraction')
    assert np.abs(g - gc).max() <= 1e-11 * np.abs(gc).max()
    ex = exponents_of(mol)
    fprims = [p for p, (sh, _) in enumerate((i, k) for i in range(mol.nbas)
                                            for k in range(mol.bas[i, M.NPRIM_OF]))
              if mol.bas[sh, M.ANG_OF] == 3]
    for p in fprims[:3]:
        hp = 1e-5 * ex[p]
        ep, em = ex.copy(), ex.copy()
        ep[p] += hp
        em[p] -= hp
        Ep = float(CoulombPlans(with_geometry(mol, exps=ep)).energy(dmt)[0])
        Em = float(CoulombPlans(with_geometry(mol, exps=em)).energy(dmt)[0])
        fd = (Ep - Em) / (2 * hp)
        assert abs(fd - ga[p]) <= 1e-7 * max(1.0, abs(ga[p])), (p, fd, ga[p])


def test_adjoint_c4_geometry_matches_ip1(gpulib):
    """c4-type bases (s..g shells, 1-8 primitives, atoms 2-5 bohr apart): 4000 sampled unique
    quartets through the contraction-first adjoint and through int2e_ip1 formed on the GPU and
    contracted, agreeing to 1e-10 of the largest gradient element (distant pairs of a tight and a
    diffuse shell are where carrying the density through the transfer loses precision)."""
    import torch
    from libcint_gb300.coulomb import CoulombPlans, IP1Gradient
    mol = M.config4(seed=2, natm=4, box=5.2)
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    rng = np.random.RandomState(9)
    d = rng.normal(0, 0.1, (nao, nao))
    dmt = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    q = np.asarray(M.unique_quartets(mol.nbas))
    q = q[rng.choice(len(q), 4000, replace=False)]
    g = CoulombPlans(mol, q).grad(dmt)[0]
    route = IP1Gradient(mol, q)
    gi = route.grad(dmt)
    route.close()
    err = float((g - gi).abs().max() / gi.abs().max())
    assert err <= 1e-10, err
