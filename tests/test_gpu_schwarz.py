"""The Schwarz-surviving quartet list from the GPU's own bounds equals libcint's.

Q_ij = sqrt(max |(ab|ab)|) from one GPU int2e_sph plan over the diagonal quartets
(libcint_gb300.screening.pair_bounds) for the 38k shell pairs of a 20000-quartet uniform sample of
c1, against libcint's own values and decisions Q_ij Q_kl >= 1e-12 (tests/golden/c1_schwarz.npz,
made by tests/golden/make_schwarz_sample.py from libcint's int2e_sph), the rule the benchmark list
was screened with.  The decisions must agree exactly.  The bounds agree to 1e-6 relative: the
diagonal blocks of distant f-f pairs with very different exponents are ill-conditioned (the
horizontal transfer builds them from moments about a distant centre), and libcint, which puts the
second shell of an equal-l pair at the recurrence base, is ~3e-7 off on some of them; the GPU
orients such pairs by exponent and is checked against the long-double referee at 1e-9 on the f-f
pairs and a sample of the others."""
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M

pytestmark = pytest.mark.gpu

THRESHOLD = 1e-12


def test_c1_schwarz_list_matches_libcint(gpulib, oracle):
    from libcint_gb300.screening import pair_bounds
    fx = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_schwarz.npz'))
    mol = M.config1(seed=0)
    pairs, qref = fx['pairs'], fx['q']
    q = pair_bounds(mol, pairs)
    err = np.abs(q - qref)
    bad = np.nonzero(err > 1e-6 * qref + 1e-15)[0]
    assert not len(bad), [(pairs[b].tolist(), float(q[b]), float(qref[b])) for b in bad[:8]]
    assert ((q == 0) == (qref == 0)).all()
    pos = {(int(a), int(b)): t for t, (a, b) in enumerate(pairs)}
    quartets = fx['quartets']
    qa = q[[pos[(int(x[0]), int(x[1]))] for x in quartets]]
    qb = q[[pos[(int(x[2]), int(x[3]))] for x in quartets]]
    keep = qa * qb >= THRESHOLD
    # the same surviving list: every decision agrees (no product lies within 1e-6 of the
    # threshold in this sample, so the bounds' agreement decides every case)
    assert not (np.abs(qa * qb / THRESHOLD - 1) < 1e-6).any()
    assert (keep == fx['keep']).all(), int((keep != fx['keep']).sum())
    assert 1000 < keep.sum() < len(keep)
    # the bounds themselves against the referee: 60 f-f pairs and 200 others
    L = mol.bas[:, 1]
    ff = np.nonzero((L[pairs[:, 0]] == 3) & (L[pairs[:, 1]] == 3) & (qref > 0))[0][:60]
    other = np.random.RandomState(2).choice(np.nonzero(qref > 0)[0], 200, replace=False)
    sel = np.concatenate([ff, other])
    items = np.concatenate([pairs[sel], pairs[sel]], 1).astype(np.int32)
    ref, offs = oracle.referee('int2e_sph', mol, items)
    qr = np.array([np.sqrt(np.abs(ref[offs[t]:offs[t + 1]]).max()) for t in range(len(sel))])
    rel = np.abs(q[sel] - qr) / qr
    assert rel.max() <= 1e-9, (pairs[sel[np.argmax(rel)]].tolist(), float(rel.max()))
