"""The symmetry algebra of the J/K contraction kernels, on the CPU against the oracle's ERIs.

The contraction kernels visit each 8-fold unique shell quartet once, in the kernel's shell order
(a b|c d) (larger l first within each pair, the larger pair first), and add contractions of its
block into accumulators that the caller symmetrises:

* J:  X[a,b] += s_cd (ab|cd) D[c,d];  X[c,d] += s_ab (ab|cd) D[a,b] if ab != cd  (s = 2 for a
      pair of two different shells);  J = X + X^T - (shell-diagonal blocks of X);
* K:  X[a,c] += w (ab|cd) D[b,d],  X[b,c] += w (ab|cd) D[a,d],  X[a,d] += w (ab|cd) D[b,c],
      X[b,d] += w (ab|cd) D[a,c]  (w halves for each coincidence a = b, c = d, ab = cd);
      K = X + X^T.

This file restates both schemes in numpy on spherical blocks from the oracle and checks them
against J = einsum('ijkl,kl->ij') and K = einsum('ijkl,jl->ik') of the full ERI tensor, for
the unique list as given and in the kernel's shell order, with one- and two-column
contractions.  The GPU tests check the kernels against the same einsums."""
import numpy as np

from libcint_gb300 import molecules as M


def _basis():
    """3 atoms; s, p, d shells, one d shell with two contraction columns, one p with one primitive."""
    rng = np.random.RandomState(5)
    b = M._Builder()
    xyz = [(0.0, 0.0, 0.0), (1.3, -0.4, 0.9), (-0.8, 1.5, 0.2)]
    for a, x in enumerate(xyz):
        at = b.atom(a + 1, x)
        b.shell(at, 0, [3.1, 0.6], [M.gto_norm(0, 3.1) * 0.7, M.gto_norm(0, 0.6) * 0.4])
        b.shell(at, 1, [0.9], [M.gto_norm(1, 0.9)])
        if a != 1:
            ex = [2.2, 0.5]
            cols = rng.uniform(0.2, 1.0, (2, 2))
            b.shell(at, 2, ex, [[M.gto_norm(2, e) * c for e, c in zip(ex, col)] for col in cols], nctr=2)
    return b.mol('jk-algebra')


def _eri_full(oracle, mol):
    loc = mol.ao_loc()
    n = loc[-1]
    eri = np.zeros((n, n, n, n))
    blocks = {}
    for q in M.unique_quartets(mol.nbas):
        i, j, k, l = (int(x) for x in q)
        _, blk = oracle.port.call('int2e_sph', mol, (i, j, k, l))
        blocks[(i, j, k, l)] = blk
        for (a, b, c, d, t) in ((i, j, k, l, 'ijkl'), (j, i, k, l, 'jikl'), (i, j, l, k, 'ijlk'),
                                (j, i, l, k, 'jilk'), (k, l, i, j, 'klij'), (l, k, i, j, 'lkij'),
                                (k, l, j, i, 'klji'), (l, k, j, i, 'lkji')):
            eri[loc[a]:loc[a + 1], loc[b]:loc[b + 1], loc[c]:loc[c + 1], loc[d]:loc[d + 1]] = \
                np.transpose(blk, ['ijkl'.index(ch) for ch in t])
    return eri, blocks


def _kernel_order(mol, q):
    """The shell order the plan builder gives the kernels (a permutation of the unique quartet)."""
    L = mol.bas[:, M.ANG_OF]
    a, b, c, d = q
    if L[a] < L[b]:
        a, b = b, a
    if L[c] < L[d]:
        c, d = d, c
    if L[a] * 16 + L[b] < L[c] * 16 + L[d]:
        a, b, c, d = c, d, a, b
    return a, b, c, d


def _contract(mol, blocks, dm, kernel_order):
    loc = mol.ao_loc()
    n = loc[-1]
    XJ, XK = np.zeros((n, n)), np.zeros((n, n))
    diag = np.zeros((n, n), dtype=bool)
    for i in range(mol.nbas):
        diag[loc[i]:loc[i + 1], loc[i]:loc[i + 1]] = True
    for q, blk in blocks.items():
        if kernel_order:
            o = _kernel_order(mol, q)
            blk = _permute_block(blk, q, o)
            q = o
        a, b, c, d = q
        sa, sb, sc, sd = (slice(loc[x], loc[x + 1]) for x in q)
        # sym flags as the host sets them: bit0 a != b, bit1 c != d, bit2 {a,b} != {c,d}
        sym = (a != b) | ((c != d) << 1) | (((min(a, b), max(a, b)) != (min(c, d), max(c, d))) << 2)
        s_ab = 2.0 if sym & 1 else 1.0
        s_cd = 2.0 if sym & 2 else 1.0
        XJ[sa, sb] += s_cd * np.einsum('abcd,cd->ab', blk, dm[sc, sd])
        if sym & 4:
            XJ[sc, sd] += s_ab * np.einsum('abcd,ab->cd', blk, dm[sa, sb])
        w = (1.0 if sym & 1 else 0.5) * (1.0 if sym & 2 else 0.5) * (1.0 if sym & 4 else 0.5)
        XK[sa, sc] += w * np.einsum('abcd,bd->ac', blk, dm[sb, sd])
        XK[sb, sc] += w * np.einsum('abcd,ad->bc', blk, dm[sa, sd])
        XK[sa, sd] += w * np.einsum('abcd,bc->ad', blk, dm[sb, sc])
        XK[sb, sd] += w * np.einsum('abcd,ac->bd', blk, dm[sa, sc])
    J = XJ + XJ.T - np.where(diag, XJ, 0.0)
    K = XK + XK.T
    return J, K


def _permute_block(blk, q, o):
    """Block of quartet o (a permutation of q by the 8-fold symmetry) from the block of q."""
    i, j, k, l = q
    for (perm, t) in (((i, j, k, l), 'ijkl'), ((j, i, k, l), 'jikl'), ((i, j, l, k), 'ijlk'),
                      ((j, i, l, k), 'jilk'), ((k, l, i, j), 'klij'), ((l, k, i, j), 'lkij'),
                      ((k, l, j, i), 'klji'), ((l, k, j, i), 'lkji')):
        if perm == tuple(o):
            return np.transpose(blk, ['ijkl'.index(ch) for ch in t])
    raise AssertionError('%s is not a permutation of %s' % (o, q))


def test_jk_schemes_match_full_tensor(oracle):
    mol = _basis()
    eri, blocks = _eri_full(oracle, mol)
    n = eri.shape[0]
    rng = np.random.RandomState(2)
    d = rng.normal(0, 0.3, (n, n))
    dm = 0.5 * (d + d.T)
    Jref = np.einsum('ijkl,kl->ij', eri, dm)
    Kref = np.einsum('ijkl,jl->ik', eri, dm)
    for kernel_order in (False, True):
        J, K = _contract(mol, blocks, dm, kernel_order)
        assert np.abs(J - Jref).max() <= 1e-12 * np.abs(Jref).max()
        assert np.abs(K - Kref).max() <= 1e-12 * np.abs(Kref).max()
    # the exchange energy -1/4 tr(D K) is the same contraction read the other way
    assert abs(np.einsum('ij,ij', dm, Kref) - np.einsum('ijkl,ik,jl', eri, dm, dm)) \
        <= 1e-12 * abs(np.einsum('ij,ij', dm, Kref))
