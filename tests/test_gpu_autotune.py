"""The autotuner on the GPU (libcint_gb300/autotune.py): every launch candidate is timed on a real
plan and the heaviest classes in both task groups, the choice is stored in the cache file and read
back without re-timing, and the tuned plan's integrals are the default plan's within 1e-13 of the
block scale (the candidates change only shared memory per warp, hence terms per batch and
summation order, the group a class runs in, and where finished quartets are transformed)."""
import json

import numpy as np
import pytest

import libcint_gb300 as cg
from libcint_gb300 import autotune
from libcint_gb300 import molecules as M
from tests import c1_sample

pytestmark = pytest.mark.gpu


def test_tune_on_gpu_caches_and_matches_default(gpulib, tmp_path):
    import torch
    mol = M.config1(seed=0)
    qs = np.ascontiguousarray(c1_sample.c1_quartets()[:3000], dtype=np.int32)
    path = str(tmp_path / 'tuning.json')
    best = autotune.choose(cg.INT2E_SPH, mol, qs, path=path, class_tuner=autotune.tune_classes)
    entries = json.load(open(path))['entries']
    assert len(entries) == 1
    (entry,) = entries.values()
    assert len(entry['ms']) == len(autotune.CANDIDATES)
    assert all(t > 0 for t in entry['ms'].values())
    assert '%d,%d' % best[:2] == min(entry['ms'], key=entry['ms'].get)
    # per class: the heaviest classes timed in both groups; the kept set is a subset of them
    assert entry['class_ms'] and all(a > 0 and b > 0 for a, b in entry['class_ms'].values())
    assert set(best[2]) <= set(int(k) for k in entry['class_ms'])

    def no_tuning(*a, **k):
        raise AssertionError('the cached choice must be used')
    assert autotune.choose(cg.INT2E_SPH, mol, qs, path=path, tuner=no_tuning,
                           class_tuner=no_tuning) == best

    ref = cg.Plan(cg.INT2E_SPH, mol, qs)
    a = torch.empty(ref.output_size, dtype=torch.float64, device='cuda')
    ref.execute(a)
    tp = autotune.tuned_plan(cg.INT2E_SPH, mol, qs, path=path)
    b = torch.empty(tp.output_size, dtype=torch.float64, device='cuda')
    tp.execute(b)
    torch.cuda.synchronize()
    ref.close()
    tp.close()
    assert torch.abs(a - b).max().item() <= 1e-13 * torch.abs(a).max().item()
