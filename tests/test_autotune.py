"""The launch-parameter autotuner's host logic on the CPU: workload keys, the cache file (missing,
damaged, foreign, merged, written atomically), candidate selection with an injected timer, cache
hits without tuning; and the C side: cintgpu_plan_create_tuned's argument checks and the shared
memory per warp reaching the planner."""
import ctypes
import json
import os

import numpy as np

from tests import _oracle  # noqa: F401  (puts the repo root on sys.path)
import libcint_gb300 as cg
from libcint_gb300 import autotune as at
from libcint_gb300 import molecules as M


def _c0():
    mol = M.config0(seed=1)
    return mol, M.unique_quartets(mol.nbas)[:500]


def test_workload_key_is_stable_and_discriminating():
    mol, qs = _c0()
    k = at.workload_key(cg.INT2E_SPH, mol, qs)
    perm = qs[np.random.RandomState(0).permutation(len(qs))]
    assert at.workload_key(cg.INT2E_SPH, mol, perm) == k                  # order-free
    swapped = qs[:, [1, 0, 3, 2]]                                          # same classes
    assert at.workload_key(cg.INT2E_SPH, mol, swapped) == k
    assert at.workload_key(cg.INT2E_CART, mol, qs) != k                   # kind
    assert at.workload_key(cg.INT2E_SPH, mol, qs[:20]) != k               # length magnitude
    L = mol.bas[:, M.ANG_OF]
    dd = qs[(L[qs] == 2).all(1)]
    assert len(dd) > 0 and at.workload_key(cg.INT2E_SPH, mol, np.tile(dd, (40, 1))[:500]) != k
    prof = at.class_profile(mol, qs)
    assert abs(sum(prof.values()) - 1.0) < 0.05
    assert all(len(c.split(',')) == 4 for c in prof if c != 'rest')


def test_cache_file_robustness(tmp_path):
    p = str(tmp_path / 'sub' / 'tuning.json')
    assert at.load_cache(p) == {}                                          # missing
    at.store('a', (16, 0), {(16, 0): 1.5, (24, 0): 2.0}, p)
    at.store('b', (24, 1), None, p)                                        # merged
    e = at.load_cache(p)
    assert e['a']['ws_kb'] == 16 and e['a']['ms']['16,0'] == 1.5 and e['b']['separate_output'] == 1
    assert [f for f in os.listdir(os.path.dirname(p)) if f.endswith('.tmp')] == []
    with open(p, 'w') as f:
        f.write('{not json')
    assert at.load_cache(p) == {}                                          # damaged
    with open(p, 'w') as f:
        json.dump({'format': 99, 'entries': {'a': {'ws_kb': 16, 'separate_output': 0}}}, f)
    assert at.load_cache(p) == {}                                          # foreign format
    with open(p, 'w') as f:
        json.dump({'format': at.FORMAT, 'entries': {'a': {'ws_kb': 99, 'separate_output': 0},
                                                    'b': {'ws_kb': 20, 'separate_output': 0}}}, f)
    assert list(at.load_cache(p)) == ['b']                                 # invalid entry dropped
    at.store('c', (32, 0), None, p)                                        # rewrite over it
    assert sorted(at.load_cache(p)) == ['b', 'c']


class _FakePlan:
    closed = 0

    def __init__(self, ws, sep):
        self.ws, self.sep = ws, sep

    def close(self):
        _FakePlan.closed += 1


def test_tune_picks_the_fastest_and_closes_every_plan():
    mol, qs = _c0()
    ms = {(24, 0): 3.0, (16, 0): 2.5, (20, 0): 2.2, (32, 0): 4.0, (24, 1): 3.1}
    _FakePlan.closed = 0
    best, times = at.tune(cg.INT2E_SPH, mol, qs, make_plan=_FakePlan,
                          timer=lambda p: ms[(p.ws, p.sep)])
    assert best == (20, 0) and times == ms and _FakePlan.closed == len(at.CANDIDATES)


def test_choose_uses_the_cache_before_tuning(tmp_path):
    mol, qs = _c0()
    p = str(tmp_path / 'tuning.json')
    calls = []

    def tuner(kind, mol_, items):
        calls.append(kind)
        return (16, 1), {(16, 1): 1.0}
    dev = 'GB300 test|cuda 13.0'
    assert at.choose(cg.INT2E_SPH, mol, qs, p, device=dev, tuner=tuner) == (16, 1, ())
    assert at.choose(cg.INT2E_SPH, mol, qs, p, device=dev, tuner=tuner) == (16, 1, ())
    assert len(calls) == 1                                                  # second call: hit
    at.choose(cg.INT2E_SPH, mol, qs, p, device='other GPU|cuda 13.0', tuner=tuner)
    assert len(calls) == 2                                                  # keyed by device
    at.choose(cg.INT2E_SPH, mol, qs, p, retune=True, device=dev, tuner=tuner)
    assert len(calls) == 3


def test_tuned_create_checks_its_arguments():
    L = cg.lib()
    mol, qs = _c0()
    items = np.ascontiguousarray(qs[:4], dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    h = ctypes.c_void_p()
    for ws, sep in ((4, 0), (64, 0), (24, 2)):
        rc = L.cintgpu_plan_create_tuned(ctypes.byref(h), cg.INT2E_SPH, P(items), 4, None,
                                         P(mol.atm), mol.natm, P(mol.bas), mol.nbas, P(mol.env),
                                         ws, sep)
        assert rc == -1 and not h.value
        assert 'ws_kb' in cg.last_error() or 'separate_output' in cg.last_error()


def test_shared_memory_per_warp_reaches_the_planner():
    """ws_kb sets the regular group's doubles per warp (0 = the default 24 KB); with 8 KB the
    (ii|ii)-type classes of an l = 6 basis no longer fit it and move to the 48 KB group."""
    from tests.test_gpu_high_l import high_l_basis
    f = cg.lib().cg_plan_groups_ws
    f.restype = ctypes.c_int
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)

    def plan_info(mol, qs, ws):
        items = np.ascontiguousarray(qs, dtype=np.int32)
        info = np.zeros(5, np.int64)
        assert f(cg.INT2E_SPH, P(items), ctypes.c_int64(len(items)), P(mol.atm), mol.natm,
                 P(mol.bas), mol.nbas, P(mol.env), ws, P(info)) == 0, cg.last_error()
        return info
    mol = M.config1(seed=0)
    qs = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_quartets.npz'))['quartets'][:400]
    res = {ws: plan_info(mol, qs, ws) for ws in (0, 8, 16, 24, 32)}
    assert (res[0] == res[24]).all() and res[0][4] == 24 * 1024 // 8
    assert all(res[ws][4] == ws * 1024 // 8 for ws in (8, 16, 32))
    hl = high_l_basis()
    big = [(0, 0, 0, 0), (1, 1, 1, 1), (2, 2, 2, 2)]
    assert plan_info(hl, big, 24)[1] == 0 and plan_info(hl, big, 8)[1] > 0


def test_tune_classes_marks_the_classes_the_wide_group_speeds_up():
    """Per-class tuning with stand-in timings of the whole list: a class goes to the 48 KB group
    when the list is faster with it there, not when it is slower; the choice is cached with the
    launch parameters."""
    mol, qs = _c0()
    keys, w = at.kernel_classes(mol, qs)
    uk = np.unique(keys)
    assert len(uk) > 3 and w.min() > 0
    fast = int(uk[np.argmax([w[keys == k].sum() for k in uk])])   # the heaviest class
    made = []

    class P:
        def __init__(self, lst, wide):
            self.n, self.wide = len(lst), tuple(wide)
            made.append(self)

        def close(self):
            pass

    def timer(p):
        # the heaviest class runs 20 % faster in the wide group, every other class 10 % slower
        base = float(p.n)
        return base * (0.8 if fast in p.wide else (1.1 if p.wide else 1.0))
    wide, times = at.tune_classes(cg.INT2E_SPH, mol, qs, make_plan=P, timer=timer)
    assert wide == (fast,) and times[fast][1] < times[fast][0]
    assert all(t1 > t0 for k, (t0, t1) in times.items() if k != fast)
    assert all(p.n == len(qs) for p in made)            # every timing is of the whole list
    # no class helps: nothing marked
    wide, _ = at.tune_classes(cg.INT2E_SPH, mol, qs, make_plan=P,
                              timer=lambda p: float(p.n) * (1.1 if p.wide else 1.0))
    assert wide == ()
    # two classes help alone but not together: the better one is kept
    second = int(uk[np.argsort([-w[keys == k].sum() for k in uk])[1]])

    def timer2(p):
        if len(p.wide) > 1:
            return 2.0 * p.n
        return float(p.n) * {fast: 0.8, second: 0.9}.get(p.wide[0] if p.wide else None, 1.0)
    wide, _ = at.tune_classes(cg.INT2E_SPH, mol, qs, make_plan=P, timer=timer2, min_share=0.0)
    assert wide == (fast,)
    dev = 'GB300 test|cuda 13.0'
    path = None

    def ct(kind, mol_, items, ws, sep):
        return (fast,), {fast: (2.0, 1.5)}
    import tempfile, os
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, 'tuning.json')
        got = at.choose(cg.INT2E_SPH, mol, qs, path, device=dev,
                        tuner=lambda k, m, i: ((24, 0), {(24, 0): 1.0}), class_tuner=ct)
        assert got == (24, 0, (fast,))
        entry = list(at.load_cache(path).values())[0]
        assert entry['wide'] == [fast] and entry['class_ms'][str(fast)] == [2.0, 1.5]


def test_wide_classes_move_to_the_48kb_group():
    """cintgpu_plan_create_classes's class list reaches the planner: the named class's tasks move
    from the regular group to the 48 KB one; a bad key is rejected."""
    mol, qs = _c0()
    keys, _ = at.kernel_classes(mol, qs)
    f = cg.lib().cg_plan_groups_wide
    f.restype = ctypes.c_int
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    items = np.ascontiguousarray(qs[:400], dtype=np.int32)
    k = int(keys[0])
    n_k = int((keys[:400] == k).sum())

    def info(wide):
        wa = np.ascontiguousarray(wide, dtype=np.int32)
        out = np.zeros(3, np.int64)
        assert f(cg.INT2E_SPH, P(items), ctypes.c_int64(len(items)), P(mol.atm), mol.natm,
                 P(mol.bas), mol.nbas, P(mol.env), P(wa), len(wa), P(out)) == 0, cg.last_error()
        return out
    a, b = info([]), info([k])
    assert a[1] == 0 and b[1] > 0 and a[0] + a[1] == b[0] + b[1] and n_k > 0
    h = ctypes.c_void_p()
    bad = np.array([5000], dtype=np.int32)
    rc = cg.lib().cintgpu_plan_create_classes(ctypes.byref(h), cg.INT2E_SPH, P(items), 4, None,
                                              P(mol.atm), mol.natm, P(mol.bas), mol.nbas,
                                              P(mol.env), 0, 0, P(bad), 1)
    assert rc == -1 and 'class key' in cg.last_error() and not h.value
