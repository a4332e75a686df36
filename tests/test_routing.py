"""Task routing of the planner, CPU only (host planning, no device): int2e classes whose horizontal
transfer after contraction would lose precision go elsewhere: kernel-order ll >= 4 to the
per-primitive group when its g arrays fit, lj >= 2 with li + lj >= 5 and ll <= 3 to the
bra-per-term tables of the regular groups ((dd| stays contraction first); CINTGPU_PER_PRIMITIVE_L
and CINTGPU_BRA_TERM_L move the thresholds; plans
transform their outputs inside the integral kernel."""
import ctypes
import os

import numpy as np

from tests import _oracle  # noqa: F401  (puts the repo root on sys.path)
import libcint_gb300 as cg
from libcint_gb300 import molecules as M
from tests.test_gpu_high_l import high_l_basis


def groups(kind, mol, items, env=None):
    f = cg.lib().cg_plan_groups
    f.restype = ctypes.c_int
    info = np.zeros(8, np.int64)
    items = np.ascontiguousarray(items, dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    old = {k: os.environ.get(k) for k in (env or {})}
    os.environ.update(env or {})
    try:
        rc = f(kind, P(items), ctypes.c_int64(len(items)), P(mol.atm), mol.natm, P(mol.bas),
               mol.nbas, P(mol.env), P(info))
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    assert rc == 0, cg.last_error()
    return info


def test_high_l_routing():
    mol = high_l_basis()      # shells 0..4: l = 6, 5, 4, 2, 0
    # (ih|ih): lj = ll = 5 -> per primitive; its g arrays (1764 per axis) fit the 48 KB warp
    assert groups(cg.INT2E_SPH, mol, [(0, 1, 0, 1)])[2] > 0
    # (ii|ii): per-primitive g arrays (2401 per axis) do not fit -> contraction first
    g = groups(cg.INT2E_SPH, mol, [(0, 0, 0, 0)])
    assert g[2] == 0 and g[0] + g[1] > 0
    # (dd|ss)-type and (is|ss): lj, ll < 4 -> contraction first
    g = groups(cg.INT2E_SPH, mol, [(3, 3, 4, 4), (0, 4, 4, 4)])
    assert g[2] == 0


def test_threshold_switch_and_fusion():
    mol = M.config1(seed=0)
    qs = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_quartets.npz'))['quartets']
    L = mol.bas[:, M.ANG_OF]
    ff = qs[(np.minimum(L[qs[:, 0]], L[qs[:, 1]]) == 3) | (np.minimum(L[qs[:, 2]], L[qs[:, 3]]) == 3)]
    K = np.stack([np.maximum(L[ff[:, 0]], L[ff[:, 1]]), np.minimum(L[ff[:, 0]], L[ff[:, 1]]),
                  np.maximum(L[ff[:, 2]], L[ff[:, 3]]), np.minimum(L[ff[:, 2]], L[ff[:, 3]])], 1)
    ket_ff = (K[:, 1] == 3) & (K[:, 3] == 3)            # (ff|ff)
    ff = np.concatenate([ff[~ket_ff][:40], ff[ket_ff][:10]])
    ket_ff = np.arange(len(ff)) >= 40
    g = groups(cg.INT2E_SPH, mol, ff)
    assert g[2] == 0 and g[4] == g[0] + g[1] > 0 and g[3] == 1   # bra per term, fused output
    g = groups(cg.INT2E_SPH, mol, ff[ket_ff], {'CINTGPU_PER_PRIMITIVE_L': '3'})
    assert g[2] > 0 and g[0] + g[1] == 0 and g[4] == 0  # ll >= 3: both transfers per primitive
    g = groups(cg.INT2E_SPH, mol, ff, {'CINTGPU_BRA_TERM_L': '99', 'CINTGPU_PER_PRIMITIVE_L': '4'})
    assert g[2] == 0 and g[4] == 0          # the former default: f-f transfers contraction first
    g = groups(cg.INT2E_SPH, mol, ff, {'CINTGPU_BRA_TERM_L': '99', 'CINTGPU_PER_PRIMITIVE_L': '3'})
    assert g[0] + g[1] == 0 and g[2] > 0    # all of them per primitive
    g = groups(cg.INT2E_SPH, mol, qs[:200], {'CINTGPU_PER_PRIMITIVE_L': '0'})
    assert g[0] + g[1] == 0 and g[2] > 0    # every class per primitive
    g = groups(cg.INT2E_SPH, mol, qs[:200], {'CINTGPU_SEPARATE_OUTPUT': '1'})
    assert g[3] == 1                        # the switch is read at plan creation, not here
    # int2e_ip1 never uses the contraction-first groups' tables but keeps the regular groups
    g = groups(cg.INT2E_IP1_SPH, mol, qs[:100])
    assert g[2] == 0 and g[0] + g[1] > 0


def _build(kind, mol, items):
    f = cg.lib().cg_plan_groups
    f.restype = ctypes.c_int
    info = np.zeros(4, np.int64)
    items = np.ascontiguousarray(items, dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    return f(kind, P(items), ctypes.c_int64(len(items)), P(mol.atm), mol.natm, P(mol.bas),
             mol.nbas, P(mol.env), P(info))


def _variant(mol, arr, idx, val):
    atm, bas, env = mol.atm.copy(), mol.bas.copy(), mol.env.copy()
    {'atm': atm, 'bas': bas, 'env': env}[arr][idx] = val
    return M.Mol(atm, bas, env, mol.name)


def test_invalid_input_is_rejected_with_a_message():
    """The planner's argument checks (the drop-in returns 0 with a zero block on these, the plan
    API the status): libcint asserts or exits on such input, this library never aborts."""
    mol = M.config0(seed=1)
    q = [(3, 1, 2, 0)]
    assert _build(cg.INT2E_SPH, mol, q) == 0
    cases = [
        ('negative shell', mol, [(-1, 1, 2, 0)], -1, 'negative shell'),
        ('l = 7', _variant(mol, 'bas', (3, M.ANG_OF), 7), q, -3, 'angular momentum'),
        ('nprim = 65', _variant(mol, 'bas', (3, M.NPRIM_OF), 65), q, -1, 'nprim'),
        ('atom out of range', _variant(mol, 'bas', (3, M.ATOM_OF), 99), q, -1, 'atom'),
        ('omega = NaN', _variant(mol, 'env', 8, float('nan')), q, -1, 'not finite'),
        ('NaN coordinate', _variant(mol, 'env', int(mol.atm[mol.bas[2, M.ATOM_OF], M.PTR_COORD]) + 1,
                                    float('nan')), q, -1, 'non-finite coordinate'),
        ('Inf exponent', _variant(mol, 'env', int(mol.bas[1, M.PTR_EXP]), float('inf')), q, -1,
         'non-finite exponent'),
        ('NaN coefficient', _variant(mol, 'env', int(mol.bas[0, M.PTR_COEFF]) + 1, float('nan')), q,
         -1, 'non-finite coefficient'),
    ]
    for what, m, items, code, text in cases:
        assert _build(cg.INT2E_SPH, m, items) == code, what
        assert text in cg.last_error(), (what, cg.last_error())
    # short range (omega < 0) and long range (omega > 0) are both accepted
    assert _build(cg.INT2E_SPH, _variant(mol, 'env', 8, -0.3), q) == 0
    assert _build(cg.INT2E_SPH, _variant(mol, 'env', 8, 0.3), q) == 0
    # adjoint limits: l <= 4; exponent adjoint: nprim <= 16
    lg = _variant(mol, 'bas', (3, M.ANG_OF), 5)
    assert _build(8, lg, q) == -3 and 'adjoint' in cg.last_error()
    # the host-buffer entry computes blocks only; J kinds go through plan_execute_j
    f = cg.lib().cintgpu_batch_host
    out = np.zeros(16)
    items = np.array(q, dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert f(7, P(out), P(items), 1, None, P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env)) == -1
    assert 'density' in cg.last_error()


def test_2c2e_and_contraction_kinds_on_the_host():
    """int2c2e plans every pair (libcint's 2c2e loop screens no primitive) on the contraction-first
    groups (no transfer: lj = ll = 0); the J, K and J/K kinds plan the same unique list and never
    transform outputs (they store none); bad int2c2e items and contraction kinds given to the
    host-buffer entry are rejected."""
    mol2, _ = M.config2(seed=1, natm=4, box=4.0)
    pairs = [(i, k) for i in range(0, mol2.nbas, 3) for k in range(0, mol2.nbas, 5)]
    for kind in (cg.INT2C2E_SPH, cg.INT2C2E_CART):
        g = groups(kind, mol2, pairs)
        assert g[2] == 0 and g[0] + g[1] >= len(pairs)
    assert _build(cg.INT2C2E_SPH, mol2, [(-1, 2)]) == -1 and 'negative shell' in cg.last_error()
    mol = M.config3(seed=2, natm=3, box=3.5)
    qs = M.unique_quartets(mol.nbas)
    tasks = [groups(kind, mol, qs)[:3].sum() for kind in (7, 10, 11)]
    assert tasks[0] == tasks[1] == tasks[2] > 0
    for kind in (7, 10, 11):
        assert groups(kind, mol, qs)[3] == 0
    f = cg.lib().cintgpu_batch_host
    out = np.zeros(16)
    items = np.array(qs[:1], dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for kind in (10, 11):
        assert f(kind, P(out), P(items), 1, None, P(mol.atm), mol.natm, P(mol.bas), mol.nbas,
                 P(mol.env)) == -1
        assert 'density' in cg.last_error()


def test_plan_image_hash_is_deterministic():
    """The planner is deterministic: the same list gives the same upload image, launch groups and
    scalars (FNV-1a hash of all of them), and a changed exponent changes it.  Changes to the
    planner's speed are checked against such hashes."""
    f = cg.lib().cg_plan_image_hash
    f.restype = ctypes.c_int
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)

    def h(mol, items, kind=cg.INT2E_SPH):
        items = np.ascontiguousarray(items, dtype=np.int32)
        out = np.zeros(1, np.uint64)
        assert f(kind, P(items), ctypes.c_int64(len(items)), P(mol.atm), mol.natm, P(mol.bas),
                 mol.nbas, P(mol.env), ctypes.c_int64(0), P(out)) == 0, cg.last_error()
        return int(out[0])
    mol = M.config0(seed=4)
    qs = M.unique_quartets(mol.nbas)[:3000]
    assert h(mol, qs) == h(mol, qs)
    assert h(mol, qs, 7) == h(mol, qs, 7)
    moved = _variant(mol, 'env', int(mol.bas[2, M.PTR_EXP]), mol.env[mol.bas[2, M.PTR_EXP]] * 1.01)
    assert h(moved, qs) != h(mol, qs)


def test_empty_lists_plan_for_every_kind():
    """n = 0 plans build (no tasks, no groups launched; the output kernel, where one runs, has
    one block and no quartets) for every kind"""
    f = cg.lib().cg_plan_groups
    f.restype = ctypes.c_int
    mol = M.config0(seed=1)
    items = np.zeros((1, 4), dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for kind in (cg.INT2E_SPH, cg.INT2E_CART, cg.INT2E_IP1_SPH, cg.INT2E_IP1_CART, cg.INT3C2E_SPH,
                 cg.INT3C2E_CART, cg.INT2C2E_SPH, cg.INT2C2E_CART, 7, 8, 9, 10, 11):
        info = np.full(4, -1, np.int64)
        assert f(kind, P(items), ctypes.c_int64(0), P(mol.atm), mol.natm, P(mol.bas), mol.nbas,
                 P(mol.env), P(info)) == 0, (kind, cg.last_error())
        assert info[:3].sum() == 0
