"""Host logic of the contraction-first int2e path, CPU only: the class tables built by the
planner (stage-3 groups, accumulator permutations, the horizontal-transfer program and its buffer
size), replayed in numpy the way the kernels use them, give the same Cartesian block as the per-term horizontal transfer
(libcint's order of operations, src/g2e.c:560-693 then src/cint2e.c:961-1183) on random VRR
arrays."""
import ctypes
import math

import numpy as np
import pytest

from tests import _oracle  # noqa: F401  (puts the repo root on sys.path)
import libcint_gb300 as cg


def nc(l):
    return (l + 1) * (l + 2) // 2


def below(l):
    return l * (l + 1) * (l + 2) // 6


def cart_list(l):
    return [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]


def tables(li, lj, lk, ll, bra=0):
    f = cg.lib().cg_eri_tables
    f.restype = ctypes.c_int
    info = np.zeros(12, np.int32)
    groups = np.zeros(4 * 200000, np.int32)
    perm = np.zeros(8000, np.int32)
    prog = np.zeros(400000, np.int32)
    rounds = np.zeros(20000, np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    nprog = f(li, lj, lk, ll, bra, P(info), P(groups), 200000, P(perm), 8000, P(prog), prog.size,
              P(rounds), rounds.size)
    assert nprog >= 0
    keys = ['group_off', 'ngroup', 'perm_off', 'nE', 'nF', 'split', 'hrr_need', 'maxab', 'hprog_off',
            'round_off', 'nround', 'bra']
    c = dict(zip(keys, info.tolist()))
    return (c, groups[:4 * c['ngroup']].reshape(-1, 4), perm[:c['nE'] + c['nF']], prog[:nprog],
            rounds[:c['nround']].astype(np.int64) & 0xffffffff)


def hrr(src, eperm, fperm, prog, li, lj, lk, ll, AB, CD, need, bra_done=False):
    """cg_hrr replayed on the class's transfer program: returns the Cartesian block in gctr order
    and checks the buffers stay within the class's hrr_need.  bra_done: rows are (i j| already."""
    bE, bF = below(li), below(lk)
    nE = nc(li) * nc(lj) if bra_done else below(li + lj + 1) - bE
    nF = below(lk + ll + 1) - bF
    cur = np.array([src[eperm[e] * nF + fperm[f]] for e in range(nE) for f in range(nF)])
    used = cur.size
    p = 0
    for b in range(1, (0 if bra_done else lj) + 1):
        nrows = prog[p]
        rows = prog[p + 1:p + 1 + 3 * nrows].reshape(-1, 3)
        nxt = np.zeros(nrows * nF)
        for r, (hi, lo, ax) in enumerate(rows):
            assert 0 <= hi * nF and (hi + 1) * nF <= cur.size and (lo + 1) * nF <= cur.size
            nxt[r * nF:(r + 1) * nF] = AB[ax] * cur[lo * nF:(lo + 1) * nF] + cur[hi * nF:(hi + 1) * nF]
        p += 1 + 3 * nrows
        cur = nxt
        used = max(used, cur.size)
    nfi, nfj, nfk, nfl = nc(li), nc(lj), nc(lk), nc(ll)
    nij = nfi * nfj
    for d in range(1, ll + 1):
        nent, sin, sout = prog[p:p + 3]
        ents = prog[p + 3:p + 3 + 3 * nent].reshape(-1, 3)
        nxt = np.zeros(nij * sout)
        for ij in range(nij):
            for q, (hi, lo, ax) in enumerate(ents):
                assert hi < sin and lo < sin
                nxt[ij * sout + q] = CD[ax] * cur[ij * sin + lo] + cur[ij * sin + hi]
        p += 3 + 3 * nent
        cur = nxt
        used = max(used, cur.size)
    assert p == len(prog)
    out = np.zeros(nij * nfk * nfl)
    for e in range(out.size):
        i, r = e % nfi, e // nfi
        k, r = r % nfk, r // nfk
        l, j = r % nfl, r // nfl
        out[e] = cur[((i * nfj + j) * nfk + k) * nfl + l]
    assert max(used, out.size) <= need
    return out


def direct(g, li, lj, lk, ll, AB, CD):
    """Per-term transfer of each axis, then the product over axes summed over terms."""
    nT, _, nm, na = g.shape
    # g4[t, ax, i, j, k, l]
    g4 = np.zeros((nT, 3, li + 1, lj + 1, lk + 1, ll + 1))
    for ax in range(3):
        # bra: h[e, j, m]
        h = np.zeros((nT, na, lj + 1, nm))
        h[:, :, 0, :] = np.transpose(g[:, ax], (0, 2, 1))
        for j in range(1, lj + 1):
            for e in range(na - j):
                h[:, e, j] = h[:, e + 1, j - 1] + AB[ax] * h[:, e, j - 1]
        for i in range(li + 1):
            for j in range(lj + 1):
                q = np.zeros((nT, nm, ll + 1))
                q[:, :, 0] = h[:, i, j, :]
                for l in range(1, ll + 1):
                    for f in range(nm - l):
                        q[:, f, l] = q[:, f + 1, l - 1] + CD[ax] * q[:, f, l - 1]
                g4[:, ax, i, j] = q[:, :lk + 1, :]
    nfi, nfj, nfk, nfl = nc(li), nc(lj), nc(lk), nc(ll)
    out = np.zeros(nfi * nfj * nfk * nfl)
    ci, cj, ck, cl = cart_list(li), cart_list(lj), cart_list(lk), cart_list(ll)
    for e in range(out.size):
        i, r = e % nfi, e // nfi
        k, r = r % nfk, r // nfk
        l, j = r % nfl, r // nfl
        v = np.ones(nT)
        for ax in range(3):
            v = v * g4[:, ax, ci[i][ax], cj[j][ax], ck[k][ax], cl[l][ax]]
        out[e] = v.sum()
    return out


CLASSES = [(0, 0, 0, 0), (1, 0, 0, 0), (1, 1, 0, 0), (1, 1, 1, 1), (2, 1, 1, 0), (2, 2, 2, 1),
           (3, 2, 2, 1), (3, 3, 2, 2), (3, 1, 3, 0), (4, 2, 3, 3), (5, 4, 1, 0), (4, 4, 4, 4)]
# plus a seeded sample of the other kernel-order classes up to f (li >= lj, lk >= ll)
_rng = np.random.RandomState(17)
_all = [(a, b, c, d) for a in range(4) for b in range(a + 1) for c in range(4) for d in range(c + 1)
        if (a, b, c, d) not in CLASSES]
CLASSES += [_all[i] for i in _rng.choice(len(_all), 16, replace=False)]


@pytest.mark.parametrize('cls', CLASSES)
def test_e0f0_tables_replay(cls):
    li, lj, lk, ll = cls
    c, groups, perm, prog, rounds = tables(*cls)
    na, nm = li + lj + 1, lk + ll + 1
    nE, nF = c['nE'], c['nF']
    assert nE == below(li + lj + 1) - below(li) and nF == below(lk + ll + 1) - below(lk)
    assert c['ngroup'] == nc(li + lj) * nc(lk + ll)
    assert c['maxab'] == (lj + 1) | ((ll + 1) << 8)
    if c['ngroup'] <= 32:
        s = c['split']
        assert s >= 1 and s & (s - 1) == 0 and s * c['ngroup'] <= 32 < 2 * s * c['ngroup']
    else:
        assert c['split'] == 0
    # every accumulator is covered by exactly one (group, member)
    hit = np.zeros(nE * nF, int)
    shapes = []
    for oxy, oz, acc, mn in groups:
        nez, nfz = mn & 0xff, (mn >> 8) & 0xff
        assert 1 <= nez <= lj + 1 and 1 <= nfz <= ll + 1
        shapes.append((nez, nfz))
        for a in range(nez):
            for b in range(nfz):
                hit[acc + a * nF + b] += 1
    assert (hit == 1).all()
    assert shapes in (sorted(shapes, reverse=True), sorted(shapes, key=lambda x: (x[1], x[0]), reverse=True))
    # rounds: contiguous, <= 32 groups, cover every group once, box = largest nez x largest nfz
    pos, cost = 0, 0
    for rd in rounds:
        start, cnt, box = rd & 0xffff, (rd >> 16) & 0xff, rd >> 24
        assert start == pos and 1 <= cnt <= 32
        ma, mb = max(x[0] for x in shapes[start:start + cnt]), max(x[1] for x in shapes[start:start + cnt])
        assert box == ((ma - 1) + 4 * (mb - 1) if ma <= 4 and mb <= 4 else 0xff)
        cost += 32 * (ma * mb + 1)
        pos += cnt
    assert pos == len(groups)
    # never worse than plain rounds of 32 in the same order
    plain = sum(32 * (max(x[0] for x in shapes[r:r + 32]) * max(x[1] for x in shapes[r:r + 32]) + 1)
                for r in range(0, len(shapes), 32))
    assert cost <= plain
    assert sorted(perm[:nE]) == list(range(nE)) and sorted(perm[nE:]) == list(range(nF))
    rng = np.random.RandomState(sum(cls))
    nT = 5
    g = rng.normal(size=(nT, 3, nm, na))
    AB, CD = rng.normal(size=3), rng.normal(size=3)
    acc = np.zeros(nE * nF)
    for oxy, oz, a0, mn in groups:
        ox, oy = oxy & 0xffff, oxy >> 16
        nez, nfz = mn & 0xff, (mn >> 8) & 0xff
        gx, gy, gz = (g[:, ax].reshape(nT, -1) for ax in range(3))
        p = gx[:, ox] * gy[:, oy]
        for a in range(nez):
            for b in range(nfz):
                acc[a0 + a * nF + b] += (p * gz[:, oz + a + na * b]).sum()
    got = hrr(acc, perm[:nE], perm[nE:], prog, li, lj, lk, ll, AB, CD, c['hrr_need'])
    ref = direct(g, li, lj, lk, ll, AB, CD)
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())


def test_all_class_tables_stay_in_bounds():
    """Every kernel-order class up to l = 6: stage-3 offsets inside the per-axis VRR arrays,
    accumulator indices inside the nE x nF slot, transfer-program sources inside the previous
    level and targets inside hrr_need (the buffers the kernels index with these tables)."""
    for li in range(7):
        for lj in range(li + 1):
            for lk in range(7):
                for ll in range(lk + 1):
                    c, groups, perm, prog, rounds = tables(li, lj, lk, ll)
                    na, nm = li + lj + 1, lk + ll + 1
                    G = na * nm
                    nE, nF = c['nE'], c['nF']
                    ox, oy = groups[:, 0] & 0xffff, groups[:, 0] >> 16
                    nez, nfz = groups[:, 3] & 0xff, (groups[:, 3] >> 8) & 0xff
                    assert ox.max() < G and oy.max() < G
                    assert (groups[:, 1] + (nez - 1) + na * (nfz - 1)).max() < G
                    assert (groups[:, 2] + (nez - 1) * nF + (nfz - 1)).max() < nE * nF
                    assert perm[:nE].max() < nE and perm[nE:].max() < nF
                    starts, cnts = rounds & 0xffff, (rounds >> 16) & 0xff
                    assert (cnts >= 1).all() and (cnts <= 32).all()
                    assert (starts + cnts).max() <= len(groups) and cnts.sum() == len(groups)
                    need = c['hrr_need']
                    assert nE * nF <= need
                    p, size = 0, nE * nF
                    for b in range(1, lj + 1):
                        nrows = prog[p]
                        rows = prog[p + 1:p + 1 + 3 * nrows].reshape(-1, 3)
                        assert rows[:, :2].max() < size // nF and set(rows[:, 2]) <= {0, 1, 2}
                        size = nrows * nF
                        assert size <= need
                        p += 1 + 3 * nrows
                    nij = nc(li) * nc(lj)
                    for d in range(1, ll + 1):
                        nent, sin, sout = prog[p:p + 3]
                        ents = prog[p + 3:p + 3 + 3 * nent].reshape(-1, 3)
                        assert ents[:, :2].max() < sin and nij * sin <= need and nij * sout <= need
                        assert sout == nent
                        p += 3 + 3 * nent
                    assert p == len(prog)


def bra_arrays(g, li, lj):
    """Per-term bra transfer of each axis's VRR array g[t, ax, f, a] (a <= li+lj): returns
    out[t, ax, (i + dI j) + dI dJ f], the layout of the kernels' bra classes."""
    nT, _, nm, na = g.shape
    dI, dJ = li + 1, lj + 1
    out = np.zeros((nT, 3, dI * dJ * nm))
    for ax in range(3):
        for f in range(nm):
            col = g[:, ax, f, :].copy()
            for i in range(dI):
                out[:, ax, i + dI * dJ * f] = col[:, i]
            for j in range(1, dJ):
                col[:, :na - j] = col[:, 1:na - j + 1] + AB_[0][ax] * col[:, :na - j]
                for i in range(dI):
                    out[:, ax, i + dI * j + dI * dJ * f] = col[:, i]
    return out


AB_ = [None]


def vrr_bra_inplace(vrr, nmax, mmax, dI, dJ, AB):
    """The memory procedure of vrr_bra_axis (rys_device.cuh) replayed on one buffer: the VRR array
    at out[a + (nmax+1) f], then columns from the highest f down through a one-column scratch,
    writing out[(i + dI j) + dI dJ f].  Every read of a VRR entry is checked to see the value the
    VRR stored (no transfer output overwrote it first)."""
    na, B = nmax + 1, dI * dJ
    size = B * (mmax + 1)
    out = np.full(size, np.nan)
    fresh = np.zeros(size, bool)
    for f in range(mmax + 1):
        out[na * f:na * f + na] = vrr[f]
        fresh[na * f:na * f + na] = True
    for m in range(mmax, -1, -1):
        assert fresh[na * m:na * m + na].all()
        col = out[na * m:na * m + na].copy()
        o = B * m
        def put(k, v):
            assert 0 <= o + k < size
            out[o + k] = v
            fresh[o + k] = False
        for i in range(dI):
            put(i, col[i])
        for j in range(1, dJ):
            col[:na - j] = col[1:na - j + 1] + AB * col[:na - j]
            for i in range(dI):
                put(i + dI * j, col[i])
    return out


@pytest.mark.parametrize('li,lj,mmax', [(3, 3, 0), (3, 3, 4), (4, 3, 2), (6, 6, 12), (3, 1, 3),
                                        (5, 4, 6), (2, 2, 4), (6, 3, 0)])
def test_bra_transfer_in_place(li, lj, mmax):
    """vrr_bra_axis's in-place order reads every VRR column before any transfer output lands on it
    and stays inside the per-axis array, and it equals the plain per-column transfer."""
    rng = np.random.RandomState(li * 100 + lj * 10 + mmax)
    nmax, dI, dJ = li + lj, li + 1, lj + 1
    vrr = rng.normal(size=(mmax + 1, nmax + 1))
    AB = 0.7
    got = vrr_bra_inplace(vrr, nmax, mmax, dI, dJ, AB)
    ref = np.zeros(dI * dJ * (mmax + 1))
    for f in range(mmax + 1):
        for i in range(dI):
            for j in range(dJ):
                ref[i + dI * j + dI * dJ * f] = sum(
                    math.comb(j, k) * AB ** (j - k) * vrr[f, i + k] for k in range(j + 1))
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)


BRA_CLASSES = [(3, 3, 0, 0), (3, 3, 1, 0), (3, 3, 2, 1), (3, 3, 2, 2), (3, 3, 3, 2), (4, 3, 2, 1),
               (4, 4, 3, 2), (3, 1, 2, 2), (2, 2, 1, 1), (5, 3, 0, 0), (3, 3, 3, 3)]


@pytest.mark.parametrize('cls', BRA_CLASSES)
def test_bra_tables_replay(cls):
    """Bra classes: the per-term bra arrays, the stage-3 groups (one (ij) row, nfz f members) and
    the ket-only transfer program reproduce the per-term transfer of both sides."""
    li, lj, lk, ll = cls
    c, groups, perm, prog, rounds = tables(*cls, bra=1)
    nfi, nfj = nc(li), nc(lj)
    nE, nF = c['nE'], c['nF']
    assert c['bra'] == 1 and nE == nfi * nfj and nF == below(lk + ll + 1) - below(lk)
    assert c['ngroup'] == nfi * nfj * nc(lk + ll)
    assert c['maxab'] == 1 | ((ll + 1) << 8)
    assert list(perm[:nE]) == list(range(nE))
    hit = np.zeros(nE * nF, int)
    for oxy, oz, acc, mn in groups:
        nez, nfz = mn & 0xff, (mn >> 8) & 0xff
        assert nez == 1 and 1 <= nfz <= ll + 1
        for b in range(nfz):
            hit[acc + b] += 1
    assert (hit == 1).all()
    rng = np.random.RandomState(sum(cls) + 3)
    nT, na, nm = 4, li + lj + 1, lk + ll + 1
    g = rng.normal(size=(nT, 3, nm, na))
    AB, CD = rng.normal(size=3), rng.normal(size=3)
    AB_[0] = AB
    gb = bra_arrays(g, li, lj)
    B = (li + 1) * (lj + 1)
    acc = np.zeros(nE * nF)
    for oxy, oz, a0, mn in groups:
        ox, oy = oxy & 0xffff, oxy >> 16
        nfz = (mn >> 8) & 0xff
        p = gb[:, 0, ox] * gb[:, 1, oy]
        for b in range(nfz):
            acc[a0 + b] += (p * gb[:, 2, oz + B * b]).sum()
    got = hrr(acc, perm[:nE], perm[nE:], prog, li, lj, lk, ll, AB, CD, c['hrr_need'], bra_done=True)
    ref = direct(g, li, lj, lk, ll, AB, CD)
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())


def test_all_bra_tables_stay_in_bounds():
    """Bra classes up to l = 6 (those the planner may route there: fewer than 65536 groups, the
    rounds' 16-bit group index): stage-3 offsets inside the per-axis g(i, j, f) arrays,
    accumulator indices inside nE x nF, the ket program inside hrr_need."""
    for li in range(7):
        for lj in range(1, li + 1):
            for lk in range(7):
                for ll in range(lk + 1):
                    if nc(li) * nc(lj) * nc(lk + ll) >= 65536:
                        continue
                    c, groups, perm, prog, rounds = tables(li, lj, lk, ll, bra=1)
                    B, nm = (li + 1) * (lj + 1), lk + ll + 1
                    G = B * nm
                    nE, nF = c['nE'], c['nF']
                    ox, oy = groups[:, 0] & 0xffff, groups[:, 0] >> 16
                    nfz = (groups[:, 3] >> 8) & 0xff
                    assert ox.max() < G and oy.max() < G
                    assert (groups[:, 1] + B * (nfz - 1)).max() < G
                    assert (groups[:, 2] + (nfz - 1)).max() < nE * nF
                    starts, cnts = rounds & 0xffff, (rounds >> 16) & 0xff
                    assert (starts + cnts).max() <= len(groups) and cnts.sum() == len(groups)
                    need = c['hrr_need']
                    assert nE * nF <= need and nc(li) * nc(lj) * nc(lk) * nc(ll) <= need
                    p, nij = 0, nc(li) * nc(lj)
                    for d in range(1, ll + 1):
                        nent, sin, sout = prog[p:p + 3]
                        ents = prog[p + 3:p + 3 + 3 * nent].reshape(-1, 3)
                        assert ents[:, :2].max() < sin and nij * sin <= need and nij * sout <= need
                        p += 3 + 3 * nent
                    assert p == len(prog)


def g_axis_replay(nmax, mmax, dI, dJ, dK, dL, b00, b10, b01, c00, c0p, AB, CD, swap):
    """g_axis (rys_device.cuh) restated in numpy: VRR about A (or B = A - AB, swap bit 0) and C
    (or D, bit 1), then the transfers towards the other centre; returns g[i, j, k, l]."""
    if swap & 1:
        c00, AB = c00 + AB, -AB
    if swap & 2:
        c0p, CD = c0p + CD, -CD
    na, nm = nmax + 1, mmax + 1
    T = np.zeros((nm, na))
    T[0, 0] = 1.0
    if mmax > 0:
        T[1, 0] = c0p
    for m in range(1, mmax):
        T[m + 1, 0] = c0p * T[m, 0] + m * b01 * T[m - 1, 0]
    for a in range(1, na):
        T[0, a] = c00 * T[0, a - 1] + ((a - 1) * b10 * T[0, a - 2] if a >= 2 else 0)
        for m in range(mmax):
            v = c0p * T[m, a] + a * b00 * T[m, a - 1]
            if m > 0:
                v += m * b01 * T[m - 1, a]
            T[m + 1, a] = v
    nb, nt = (dJ, dI) if swap & 1 else (dI, dJ)
    mb, mt = (dL, dK) if swap & 2 else (dK, dL)
    g = np.zeros((dI, dJ, dK, dL))
    col = T.copy()
    for t in range(nt):
        if t > 0:
            col[:, :na - t] = AB * col[:, :na - t] + col[:, 1:na - t + 1]
        for b in range(nb):
            i, j = (t, b) if swap & 1 else (b, t)
            tmp = col[:, b].copy()
            for u in range(mt):
                if u > 0:
                    tmp[:nm - u] = CD * tmp[:nm - u] + tmp[1:nm - u + 1]
                for v in range(mb):
                    k, l = (u, v) if swap & 2 else (v, u)
                    g[i, j, k, l] = tmp[v]
    return g


@pytest.mark.parametrize('li,lj,lk,ll', [(3, 3, 3, 3), (4, 2, 3, 1), (2, 4, 1, 3), (5, 4, 4, 2)])
def test_g_axis_base_swap(li, lj, lk, ll):
    """Running a pair's recurrences about its second centre gives the same 2D integrals."""
    rng = np.random.RandomState(li + 7 * lj)
    dI, dJ, dK, dL = li + 1, lj + 1, lk + 1, ll + 1
    b00, b10, b01 = rng.uniform(0.05, 0.4, 3)
    c00, c0p, AB, CD = rng.normal(size=4)
    ref = g_axis_replay(li + lj, lk + ll, dI, dJ, dK, dL, b00, b10, b01, c00, c0p, AB, CD, 0)
    for swap in (1, 2, 3):
        got = g_axis_replay(li + lj, lk + ll, dI, dJ, dK, dL, b00, b10, b01, c00, c0p, AB, CD, swap)
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())
