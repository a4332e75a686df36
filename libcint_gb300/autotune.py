"""Autotuner for the batched plans' launch parameters, with an on-disk cache.

The integral kernels derive every class's tile from the shared memory per warp of the task group
the class runs in: terms per batch are the most (term record + g array) slots that fit (at most
32), stage-3 rounds and split lanes follow from the class.  So the tuned parameters are the shared
memory per warp of the regular task group (`ws_kb`: more terms per batch against fewer CTAs per
SM), whether finished quartets are transformed at the integral kernel's tail or by their own
kernel (`separate_output`), and per class whether it runs in the regular group or in the 48 KB
group beside it (`wide`: the class's stage depth, i.e. terms per batch, against its warps per SM;
timed on the class's own items, kept only if the whole list gets faster).  A workload is keyed by its integral kind, the order of magnitude of its
length and its class profile (each (li, lj, lk, ll) class's share of the primitive-quartet work,
rounded), together with the GPU name and the CUDA version; the fastest candidate by device time
of a whole execution is stored in a JSON file (CINTGPU_TUNE_CACHE, default
~/.cache/cintgpu/tuning.json), written atomically and merged with what is there; an unreadable
or foreign file counts as empty.  No libcint counterpart (libcint has nothing to tune).
"""
import hashlib
import json
import os
import tempfile

import numpy as np

from .molecules import ANG_OF, NCTR_OF, NPRIM_OF

# (ws_kb, separate_output); the first is the default configuration
CANDIDATES = ((24, 0), (16, 0), (20, 0), (32, 0), (24, 1))
FORMAT = 2


def class_profile(mol, items):
    """{'li,lj,lk,ll': share} of the work of a list of shell tuples (2, 3 or 4 shells), each
    class keyed in the kernels' shell order (larger l first in a pair, the larger pair first) and
    weighted by primitive tuples x Cartesian components x contraction columns; classes below 1 %
    are pooled under 'rest'."""
    q = np.asarray(items, dtype=np.int64)
    q = q.reshape(len(q), -1) if len(q) else q.reshape(0, 4)
    L = mol.bas[:, ANG_OF].astype(np.int64)
    ls = L[q]
    if q.shape[1] == 4:
        a, b = np.maximum(ls[:, 0], ls[:, 1]), np.minimum(ls[:, 0], ls[:, 1])
        c, d = np.maximum(ls[:, 2], ls[:, 3]), np.minimum(ls[:, 2], ls[:, 3])
        swap = a * 16 + b < c * 16 + d
        ls = np.where(swap[:, None], np.stack([c, d, a, b], 1), np.stack([a, b, c, d], 1))
    per = mol.bas[:, NPRIM_OF] * ((L + 1) * (L + 2) // 2) * mol.bas[:, NCTR_OF]
    w = np.prod(per[q].astype(np.float64), axis=1)
    total = w.sum()
    prof = {}
    if total <= 0:
        return prof
    keys, inv = np.unique(ls, axis=0, return_inverse=True)
    share = np.bincount(inv.ravel(), weights=w) / total
    rest = 0.0
    for k, s in zip(keys, share):
        if s >= 0.01:
            prof[','.join(str(int(x)) for x in k)] = round(float(s), 2)
        else:
            rest += s
    if rest > 0:
        prof['rest'] = round(float(rest), 2)
    return prof


def kernel_classes(mol, items):
    """Per item, the class key ((li*8 + lj)*8 + lk)*8 + ll in the kernels' shell order (larger l
    first in a pair, the larger pair first; int3c2e: ll = 0), and the work weight of the item
    (primitive tuples x Cartesian components x contraction columns)."""
    q = np.asarray(items, dtype=np.int64)
    q = q.reshape(len(q), -1) if len(q) else q.reshape(0, 4)
    L = mol.bas[:, ANG_OF].astype(np.int64)
    ls = L[q]
    a, b = np.maximum(ls[:, 0], ls[:, 1]), np.minimum(ls[:, 0], ls[:, 1])
    if q.shape[1] == 4:
        c, d = np.maximum(ls[:, 2], ls[:, 3]), np.minimum(ls[:, 2], ls[:, 3])
        swap = a * 16 + b < c * 16 + d
        a, b, c, d = (np.where(swap, c, a), np.where(swap, d, b), np.where(swap, a, c),
                      np.where(swap, b, d))
    else:
        c, d = ls[:, 2], np.zeros_like(a)
    per = mol.bas[:, NPRIM_OF] * ((L + 1) * (L + 2) // 2) * mol.bas[:, NCTR_OF]
    w = np.prod(per[q].astype(np.float64), axis=1)
    return ((a * 8 + b) * 8 + c) * 8 + d, w


def workload_key(kind, mol, items):
    """A short stable key of the workload: kind, length order of magnitude, class profile."""
    n = len(items)
    blob = json.dumps({'kind': int(kind), 'size_log2': int(np.log2(max(n, 1))),
                       'profile': class_profile(mol, items)}, sort_keys=True)
    return hashlib.sha1(blob.encode()).hexdigest()[:16]


def device_key():
    """GPU name and CUDA version of the current device."""
    import torch
    return '%s|cuda %s' % (torch.cuda.get_device_name(), torch.version.cuda)


def cache_path(path=None):
    return path or os.environ.get('CINTGPU_TUNE_CACHE') or os.path.join(
        os.path.expanduser('~'), '.cache', 'cintgpu', 'tuning.json')


def _valid(entry):
    try:
        ws, sep = int(entry['ws_kb']), int(entry['separate_output'])
        wide = [int(k) for k in entry.get('wide', [])]
    except (KeyError, TypeError, ValueError):
        return False
    return (ws == 0 or 8 <= ws <= 48) and sep in (0, 1) and all(0 <= k < 4096 for k in wide)


def load_cache(path=None):
    """Entries of the cache file ({} when it is missing, unreadable or of another format)."""
    try:
        with open(cache_path(path)) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return {}
    if not isinstance(d, dict) or d.get('format') != FORMAT or not isinstance(d.get('entries'), dict):
        return {}
    return {k: v for k, v in d['entries'].items() if isinstance(v, dict) and _valid(v)}


def store(key, choice, times=None, path=None, wide=(), class_ms=None):
    """Record choice = (ws_kb, separate_output) and the wide classes under key, merged with the
    file's other entries; the file is replaced atomically (written to a temporary file in the
    same directory first)."""
    p = cache_path(path)
    entries = load_cache(p)
    entries[key] = {'ws_kb': int(choice[0]), 'separate_output': int(choice[1]),
                    'wide': sorted(int(k) for k in wide),
                    'ms': {'%d,%d' % c: float(t) for c, t in (times or {}).items()},
                    'class_ms': {str(k): [float(a), float(b)] for k, (a, b) in (class_ms or {}).items()}}
    d = os.path.dirname(os.path.abspath(p))
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d, prefix='.tuning.', suffix='.tmp')
    try:
        with os.fdopen(fd, 'w') as f:
            json.dump({'format': FORMAT, 'entries': entries}, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


def measure(plan, reps=3):
    """Best of reps device times (ms) of one whole execution (integral and output kernels), CUDA
    events on the launching stream after one warm-up execution."""
    import torch
    out = torch.empty(max(plan.ncomp * plan.output_size, 1), dtype=torch.float64, device='cuda')
    s = torch.cuda.current_stream()
    plan.execute(out, s)
    best = float('inf')
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        plan.execute(out, s)
        b.record(s)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def tune(kind, mol, items, candidates=CANDIDATES, make_plan=None, timer=measure):
    """Time every candidate on the list; returns (fastest candidate, {candidate: ms})."""
    if make_plan is None:
        from . import Plan

        def make_plan(ws, sep):
            return Plan(kind, mol, items, ws_kb=ws, separate_output=sep)
    times = {}
    for ws, sep in candidates:
        p = make_plan(ws, sep)
        try:
            times[(ws, sep)] = timer(p)
        finally:
            p.close()
    return min(times, key=times.get), times


def tune_classes(kind, mol, items, ws_kb=0, separate_output=0, min_share=0.02, max_classes=8,
                 make_plan=None, timer=measure, gain=0.98):
    """Per class carrying at least min_share of the list's work (largest first, at most
    max_classes): time the whole list with that class in the 48 KB group against the whole list
    with none there (a class's items timed alone mostly measure the launch tail of a short
    kernel, not the class's cost inside the full launch); a class is marked wide when the list
    is faster by more than 1 - gain.  Several marked classes are kept together only if the list
    is faster with all of them, else the single best one is kept.  Returns (wide keys,
    {key: (ms with the class in the regular group, ms with it in the 48 KB group)}), both whole
    list times.  Lists of 2-shell items are not tuned per class."""
    items = np.asarray(items)
    if items.ndim != 2 or items.shape[1] < 3 or len(items) == 0:
        return (), {}
    if make_plan is None:
        from . import Plan

        def make_plan(lst, wide):
            return Plan(kind, mol, lst, ws_kb=ws_kb, separate_output=separate_output,
                        wide_classes=wide)
    keys, w = kernel_classes(mol, items)
    total = w.sum()
    uk, inv = np.unique(keys, return_inverse=True)
    share = np.bincount(inv.ravel(), weights=w) / max(total, 1e-300)
    order = [int(uk[i]) for i in np.argsort(-share) if share[i] >= min_share][:max_classes]

    def timed(wset):
        p = make_plan(items, wset)
        try:
            return timer(p)
        finally:
            p.close()
    base = timed(())
    times, wide = {}, []
    for k in order:
        t1 = timed((k,))
        times[k] = (base, t1)
        if t1 < gain * base:
            wide.append(k)
    if len(wide) > 1 and timed(tuple(wide)) >= gain * base:
        wide = [min(wide, key=lambda k: times[k][1])]
    return tuple(wide), times


def choose(kind, mol, items, path=None, retune=False, device=None, tuner=tune, class_tuner=None):
    """(ws_kb, separate_output, wide classes) for the workload: the cached choice for this device
    and workload, else tuned now and stored (class_tuner: tune_classes, or a stand-in; None keeps
    every class in its default group)."""
    key = '%s|%s' % (device or device_key(), workload_key(kind, mol, items))
    entry = None if retune else load_cache(path).get(key)
    if entry is not None:
        return int(entry['ws_kb']), int(entry['separate_output']), tuple(entry.get('wide', ()))
    best, times = tuner(kind, mol, items)
    wide, class_ms = class_tuner(kind, mol, items, *best) if class_tuner else ((), {})
    store(key, best, times, path, wide, class_ms)
    return best[0], best[1], tuple(wide)


def tuned_plan(kind, mol, items, offsets=None, path=None, retune=False, per_class=True):
    """A Plan with the launch parameters the cache (or a tuning run) picks for this workload."""
    from . import Plan
    ws, sep, wide = choose(kind, mol, items, path, retune,
                           class_tuner=tune_classes if per_class else None)
    return Plan(kind, mol, items, offsets, ws_kb=ws, separate_output=sep, wide_classes=wide)
