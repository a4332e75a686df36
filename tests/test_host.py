"""Host-side pieces: the synthetic workloads have the sizes the benchmark configurations state,
the unique-quartet enumeration is libcint's 8-fold one, and the committed c1 sample is a valid
unique-quartet list.  CPU only."""
import os

import numpy as np

from libcint_gb300 import molecules as M


def test_config_sizes():
    c0 = M.config0(0)
    assert c0.natm == 8 and c0.nbas == 40 and c0.ao_loc()[-1] == 104
    assert len(M.unique_quartets(c0.nbas)) == 336610
    c1 = M.config1(0)
    assert c1.natm == 120 and c1.nbas == 1080 and c1.ao_loc()[-1] == 3480
    assert set(c1.bas[:, M.NPRIM_OF]) <= set(range(1, 9))
    c2, norb = M.config2(0)
    assert norb == 1000 and c2.nbas == 3000
    assert sum(c2.nsph(i) for i in range(norb)) == 2600
    assert sum(c2.nsph(i) for i in range(norb, c2.nbas)) == 10000
    c3 = M.config3(0)
    assert c3.nbas == 72 and c3.ao_loc()[-1] == 216
    c4 = M.config4(0, natm=20)
    assert c4.nbas == 200


def test_atoms_respect_min_separation():
    for mol in (M.config0(1), M.config3(2)):
        R = np.array([mol.env[mol.atm[a, M.PTR_COORD]:mol.atm[a, M.PTR_COORD] + 3] for a in range(mol.natm)])
        d = np.linalg.norm(R[:, None] - R[None], axis=-1) + np.eye(mol.natm) * 1e9
        assert d.min() >= 1.0 * M.ANGSTROM - 1e-9


def test_unique_quartets_are_eightfold_unique():
    q = M.unique_quartets(6)
    assert (q[:, 0] >= q[:, 1]).all() and (q[:, 2] >= q[:, 3]).all()
    pij = q[:, 0] * (q[:, 0] + 1) // 2 + q[:, 1]
    pkl = q[:, 2] * (q[:, 2] + 1) // 2 + q[:, 3]
    assert (pij >= pkl).all()
    assert len({tuple(r) for r in q}) == len(q) == 21 * 22 // 2


def test_c1_sample_fixture():
    qs = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_quartets.npz'))['quartets']
    assert qs.shape == (100000, 4)
    assert (qs[:, 0] >= qs[:, 1]).all() and (qs[:, 2] >= qs[:, 3]).all()
    pij = qs[:, 0].astype(np.int64) * (qs[:, 0] + 1) // 2 + qs[:, 1]
    pkl = qs[:, 2].astype(np.int64) * (qs[:, 2] + 1) // 2 + qs[:, 3]
    assert (pij >= pkl).all() and qs.max() < 1080
