"""Synthetic molecules in libcint's atm/bas/env layout.

The workloads are the five seeded systems the benchmark and the tests use (no public dataset
exists for this path; every input is generated here):

  c0  8 atoms, 6 A cube, shells s,s,p,p,d x 4 even-tempered primitives (0.15*3^k): plain int2e
  c1  120 atoms, 14 A cube, per atom 3 s, 3 p, 2 d, 1 f, 1-8 primitives, a0*beta^k exponents:
      batched int2e_sph with Schwarz screening at 1e-12 (the headline workload)
  c2  200 atoms, 18 A cube, orbital s,s,p,p,d (1-6 primitives) + auxiliary l=0..4 x 2, one
      primitive each, exponents geometric in [0.1, 20]: batched int3c2e_sph
  c3  24 atoms, 8 A cube, s,p,d with 3-5 primitives: Coulomb-like loss and its gradient
  c4  400 atoms, 24 A cube, s:3 p:3 d:2 f:1 g:1 per atom, 1-8 primitives: J-like forward and
      recomputing gradient at scale

Coordinates are in Bohr in env (1 A = 1/0.52917721092 Bohr); coefficients are u_k *
CINTgto_norm(l, alpha_k) with u_k ~ U(0.1, 1) (the scaling of libcint examples/time_c60.c:93-112);
env[PTR_EXPCUTOFF] = 0 and env[PTR_RANGE_OMEGA] = 0.  The layout constants are libcint's
(include/cint.h.in:26-72).
"""
import math

import numpy as np

ATM_SLOTS, BAS_SLOTS = 6, 8
CHARGE_OF, PTR_COORD = 0, 1
ATOM_OF, ANG_OF, NPRIM_OF, NCTR_OF, KAPPA_OF, PTR_EXP, PTR_COEFF = 0, 1, 2, 3, 4, 5, 6
PTR_ENV_START = 20
ANGSTROM = 1.0 / 0.52917721092


def gto_norm(l, a):
    """CINTgto_norm (libcint src/misc.c:72-93): 1/sqrt(int_0^inf r^(2l+2) exp(-2 a r^2) dr)."""
    n1 = (2 * l + 3) * 0.5
    return 1.0 / math.sqrt(math.gamma(n1) / (2.0 * (2 * a) ** n1))


class Mol:
    """atm/bas/env arrays plus convenience metadata."""

    def __init__(self, atm, bas, env, name=''):
        self.atm = np.ascontiguousarray(atm, dtype=np.int32)
        self.bas = np.ascontiguousarray(bas, dtype=np.int32)
        self.env = np.ascontiguousarray(env, dtype=np.float64)
        self.name = name

    @property
    def natm(self):
        return self.atm.shape[0]

    @property
    def nbas(self):
        return self.bas.shape[0]

    def l(self, sh):
        return int(self.bas[sh, ANG_OF])

    def nsph(self, sh):
        return (2 * int(self.bas[sh, ANG_OF]) + 1) * int(self.bas[sh, NCTR_OF])

    def ncart(self, sh):
        l = int(self.bas[sh, ANG_OF])
        return (l + 1) * (l + 2) // 2 * int(self.bas[sh, NCTR_OF])

    def ao_loc(self, cart=False):
        n = [self.ncart(i) if cart else self.nsph(i) for i in range(self.nbas)]
        return np.concatenate([[0], np.cumsum(n)]).astype(np.int64)

    def shell_coords(self):
        return np.array([self.env[self.atm[self.bas[i, ATOM_OF], PTR_COORD]:
                                  self.atm[self.bas[i, ATOM_OF], PTR_COORD] + 3]
                         for i in range(self.nbas)])

    def copy(self):
        return Mol(self.atm.copy(), self.bas.copy(), self.env.copy(), self.name)


class _Builder:
    def __init__(self):
        self.atm, self.bas, self.env = [], [], [0.0] * PTR_ENV_START

    def atom(self, charge, xyz_bohr):
        self.atm.append([charge, len(self.env), 1, 0, 0, 0])
        self.env.extend(float(v) for v in xyz_bohr)
        return len(self.atm) - 1

    def shell(self, atom, l, exps, coefs, nctr=1, kappa=0):
        exps = list(map(float, exps))
        coefs = list(map(float, np.asarray(coefs, dtype=float).ravel()))
        pe = len(self.env)
        self.env.extend(exps)
        pc = len(self.env)
        self.env.extend(coefs)
        self.bas.append([atom, l, len(exps), nctr, kappa, pe, pc, 0])
        return len(self.bas) - 1

    def mol(self, name):
        return Mol(np.array(self.atm).reshape(-1, ATM_SLOTS),
                   np.array(self.bas).reshape(-1, BAS_SLOTS), np.array(self.env), name)


def _place_atoms(rng, natm, box_A, min_sep_A=1.0):
    pts = []
    while len(pts) < natm:
        p = rng.uniform(0, box_A, 3)
        if all(np.linalg.norm(p - q) >= min_sep_A for q in pts):
            pts.append(p)
    return np.array(pts) * ANGSTROM


def _coefs(rng, l, exps):
    return [rng.uniform(0.1, 1.0) * gto_norm(l, a) for a in exps]


def config0(seed=0):
    """8 atoms, s,s,p,p,d x 4 primitives alpha_k = 0.15 * 3^k."""
    rng = np.random.RandomState(seed)
    b = _Builder()
    xyz = _place_atoms(rng, 8, 6.0)
    exps = [0.15 * 3 ** k for k in range(4)]
    for a in range(8):
        at = b.atom(a + 1, xyz[a])
        for l in (0, 0, 1, 1, 2):
            b.shell(at, l, exps, _coefs(rng, l, exps))
    return b.mol('c0: 8 atoms, 6 A cube, s,s,p,p,d x 4 prims')


def _even_tempered(rng, nmin, nmax):
    npr = rng.randint(nmin, nmax + 1)
    a0 = rng.uniform(0.05, 0.3)
    beta = rng.uniform(2.5, 3.5)
    return [a0 * beta ** k for k in range(npr)]


def config1(seed=0, natm=120, box=14.0):
    """120 atoms, per atom 3 s / 3 p / 2 d / 1 f shells, 1-8 primitives."""
    rng = np.random.RandomState(seed)
    b = _Builder()
    xyz = _place_atoms(rng, natm, box)
    for a in range(natm):
        at = b.atom(int(rng.randint(1, 9)), xyz[a])
        for l, cnt in ((0, 3), (1, 3), (2, 2), (3, 1)):
            for _ in range(cnt):
                exps = _even_tempered(rng, 1, 8)
                b.shell(at, l, exps, _coefs(rng, l, exps))
    return b.mol('c1: %d atoms, %g A cube, 3s3p2d1f, 1-8 prims' % (natm, box))


def config2(seed=0, natm=200, box=18.0):
    """Orbital basis (s,s,p,p,d, 1-6 primitives) and auxiliary basis (l=0..4 x 2, 1 primitive).
    Returns (mol, n_orbital_shells): orbital shells first, auxiliary shells after."""
    rng = np.random.RandomState(seed)
    b = _Builder()
    xyz = _place_atoms(rng, natm, box)
    ats = [b.atom(int(rng.randint(1, 9)), xyz[a]) for a in range(natm)]
    for at in ats:
        for l in (0, 0, 1, 1, 2):
            exps = _even_tempered(rng, 1, 6)
            b.shell(at, l, exps, _coefs(rng, l, exps))
    norb = len(b.bas)
    aux_exps = np.geomspace(0.1, 20.0, 10)
    for at in ats:
        k = 0
        for l in range(5):
            for _ in range(2):
                a = float(aux_exps[k])
                k += 1
                b.shell(at, l, [a], [gto_norm(l, a)])
    return b.mol('c2: %d atoms, %g A cube, orbital s,s,p,p,d + aux l<=4' % (natm, box)), norb


def config3(seed=0, natm=24, box=8.0):
    """24 atoms, shells s, p, d with 3-5 primitives."""
    rng = np.random.RandomState(seed)
    b = _Builder()
    xyz = _place_atoms(rng, natm, box)
    for a in range(natm):
        at = b.atom(int(rng.randint(1, 9)), xyz[a])
        for l in (0, 1, 2):
            exps = _even_tempered(rng, 3, 5)
            b.shell(at, l, exps, _coefs(rng, l, exps))
    return b.mol('c3: %d atoms, %g A cube, s,p,d x 3-5 prims' % (natm, box))


def config4(seed=0, natm=400, box=24.0):
    """400 atoms, per atom s:3 p:3 d:2 f:1 g:1, 1-8 primitives."""
    rng = np.random.RandomState(seed)
    b = _Builder()
    xyz = _place_atoms(rng, natm, box)
    for a in range(natm):
        at = b.atom(int(rng.randint(1, 9)), xyz[a])
        for l, cnt in ((0, 3), (1, 3), (2, 2), (3, 1), (4, 1)):
            for _ in range(cnt):
                exps = _even_tempered(rng, 1, 8)
                b.shell(at, l, exps, _coefs(rng, l, exps))
    return b.mol('c4: %d atoms, %g A cube, 3s3p2d1f1g, 1-8 prims' % (natm, box))


def kat_basis():
    """The self-contained basis of libcint testsuite/test_cint.py:45-140 (restated): 4 atoms,
    shells l = 1..4 (one with 2 primitives x 2 contractions) plus their l-1 copies with rescaled
    coefficients.  Returns (mol, nbas_declared) where nbas_declared = 4 is what that test passes
    to libcint while looping over all 8 shells."""
    natm = 4
    env = np.zeros(10000)
    atm = np.zeros((natm, ATM_SLOTS), np.int32)
    bas = np.zeros((8, BAS_SLOTS), np.int32)
    off = PTR_ENV_START
    for i in range(natm):
        atm[i, CHARGE_OF] = (i + 1) * 2
        atm[i, PTR_COORD] = off
        env[off:off + 3] = [.2 * (i + 1), .3 + (i + 1) * .5, .1 - (i + 1) * .5]
        off += 3
    off0 = off
    spec = [(0, 1, [1.], [1.], 1), (1, 2, [5., 3.], [1., 2., 4., 1.], 2),
            (2, 3, [1.], [1.], 1), (3, 4, [.5], [1.], 1)]
    for nh, (at, l, ex, cf, nctr) in enumerate(spec):
        bas[nh] = [at, l, len(ex), nctr, l, off, off + len(ex), 0]
        env[off:off + len(ex)] = ex
        env[off + len(ex):off + len(ex) + len(cf)] = cf
        off += len(ex) + len(cf)
    n = off - off0
    env[off:off + n] = env[off0:off0 + n]
    for i in range(4):
        bas[i + 4] = bas[i]
        bas[i + 4, ANG_OF] = bas[i, ANG_OF] - 1
        bas[i + 4, KAPPA_OF] = -bas[i, KAPPA_OF]
        bas[i + 4, PTR_EXP] = bas[i, PTR_EXP] + n
        bas[i + 4, PTR_COEFF] = bas[i, PTR_COEFF] + n
        env[bas[i + 4, PTR_COEFF]] /= 2 * env[bas[i, PTR_EXP]]
    c5, c1, e1 = bas[5, PTR_COEFF], bas[1, PTR_COEFF], bas[1, PTR_EXP]
    env[c5 + 0] = env[c1 + 0] / (2 * env[e1 + 0])
    env[c5 + 1] = env[c1 + 1] / (2 * env[e1 + 1])
    env[c5 + 2] = env[c1 + 2] / (2 * env[e1 + 0])
    env[c5 + 3] = env[c1 + 3] / (2 * env[e1 + 1])
    return Mol(atm, bas, env[:off + n + 8].copy(), 'libcint test_cint.py basis'), 4


def kat_basis_3c2e():
    """KAT basis plus the zero-exponent fitting s shell of libcint testsuite/test_3c2e.py:134-146
    (coefficient 2 sqrt(pi)); index 8.  With it, int2e_sph(i,j,k,fit) equals int3c2e_sph(i,j,k)."""
    mol, _ = kat_basis()
    env = list(mol.env)
    pe = len(env)
    env += [0.0, 2.0 * math.sqrt(math.pi)]
    bas = np.vstack([mol.bas, [[0, 0, 1, 1, 0, pe, pe + 1, 0]]]).astype(np.int32)
    return Mol(mol.atm, bas, np.array(env), 'test_3c2e.py basis'), 4


def shell_nsph(mol):
    """Real-spherical functions of every shell (all contraction columns); libcint's
    CINTcgto_spheric, with l <= 1 kept Cartesian as libcint does."""
    l = mol.bas[:, ANG_OF].astype(np.int64)
    return np.where(l > 1, 2 * l + 1, (l + 1) * (l + 2) // 2) * mol.bas[:, NCTR_OF].astype(np.int64)


def unique_quartets(nbas):
    """All 8-fold unique shell quartets i>=j, k>=l, ij>=kl (row order of libcint's time_c2h6)."""
    out = []
    pairs = [(i, j) for i in range(nbas) for j in range(i + 1)]
    for a, (i, j) in enumerate(pairs):
        for (k, l) in pairs[:a + 1]:
            out.append((i, j, k, l))
    return np.array(out, dtype=np.int32).reshape(-1, 4)
