"""Benchmark of the batched Rys int2e_sph path on the c1 workload (see libcint_gb300/molecules.py).

Workload (one "step"): one execution of a batched int2e_sph plan over a seeded sample of the
Schwarz-surviving unique shell quartets of c1 (120 atoms, 14 A cube, 3s3p2d1f per atom, 1-8
primitives; keep Q_ij * Q_kl >= 1e-12 with Q_ij = sqrt(max|(ij|ij)|)).  The sample (100k
quartets, tests/golden/c1_quartets.npz) was drawn uniformly from the unique quartets
(i>=j, k>=l, ij>=kl) by rejection on libcint's own Schwarz bounds; the full list (~3e10 quartets)
does not fit a bench step.  GPU and CPU legs evaluate the same list.  Metric: spherical integrals per second
(sum of di*dj*dk*dl over the step's quartets / time).

  value      device-resident inputs, one plan execution per step, CUDA events on the launching
             stream, L2 flushed (256 MiB memset) before every step outside the events.
  e2e        the one-shot host-buffer C-ABI call cintgpu_batch_host (host planning, H2D, kernels,
             D2H of every integral) per step, wall clock.
  roofline   the Rys kernels are FP64-issue bound: achieved = algorithmic FP64 flops of a launch
             (model of cintgpu_plan_flops) / the integral kernel's own duration (CUDA events the
             plan records around it on the launching stream), against the measured DFMA peak.
  cpu_baseline  the C restatement (oracle/, "port") with OpenMP on all host cores over a bounded
             sample of the same quartet list.

--impl reference times the CPU implementation of the path on the host cores (the port; libcint
itself cannot be rebuilt where its sources are absent) and prints the same metric.
Multi-GPU (torchrun): every rank evaluates the committed list (weak scaling: fixed work per GPU),
no collectives on the data path; the time is the max over ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import struct
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FP64_PEAK_TFLOPS = 1.257      # measured DFMA peak of this GB300 pool (bench.py --only fp64peak;
                              # = 2 DFMA per SM per clock x 152 SMs x 2.07 GHz)
# DRAM read + write of one integral-kernel launch per c1 quartet: 545.8 MB + 1115.7 MB for the
# step's 100k quartets (one ncu capture of that launch)
ERI_DRAM_BYTES_PER_QUARTET = (545.8e6 + 1115.7e6) / 100000
SCHWARZ = 1e-12
# one metric string for both arms, so the two lines are directly comparable
METRIC = 'int2e_sph integrals/s (c1 Schwarz-screened quartets)'
L2_FLUSH_BYTES = 256 << 20


def load_quartets(n=None):
    """The committed c1 sample (tests/golden/c1_quartets.npz, made by make_c1_sample.py with
    libcint's own Schwarz bounds): unique quartets with Q_ij Q_kl >= 1e-12, uniform."""
    qs = np.load(os.path.join(ROOT, 'tests', 'golden', 'c1_quartets.npz'))['quartets']
    return np.ascontiguousarray(qs[:n] if n else qs, dtype=np.int32)


def integrals_of(mol, qs):
    d = np.array([mol.nsph(s) for s in range(mol.nbas)], dtype=np.int64)
    return int((d[qs[:, 0]] * d[qs[:, 1]] * d[qs[:, 2]] * d[qs[:, 3]]).sum())


def write_bench_input(path, mol, qs):
    with open(path, 'wb') as f:
        f.write(struct.pack('4i', mol.natm, mol.nbas, mol.env.size, len(qs)))
        f.write(mol.atm.astype(np.int32).tobytes())
        f.write(mol.bas.astype(np.int32).tobytes())
        f.write(mol.env.astype(np.float64).tobytes())
        f.write(np.ascontiguousarray(qs, dtype=np.int32).tobytes())


def cpu_port_rate(mol, qs, threads, target_s=12.0):
    """Time the C restatement (oracle port) with OpenMP over a bounded prefix of qs."""
    subprocess.run(['make', '-s', '-C', os.path.join(ROOT, 'oracle'), 'oracle'], check=True)
    # the restatement built with the GPU kernels' root tables (the tests' oracle keeps its own
    # Stieltjes root finder): the faster of the two CPU implementations
    exe = os.path.join(ROOT, 'oracle', '_build', 'oracle_bench_fast')
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, 'in.bin')
        n = min(len(qs), 2000)
        while True:
            write_bench_input(path, mol, qs[:n])
            r = subprocess.run([exe, path, str(threads)], capture_output=True, text=True, check=True)
            res = json.loads(r.stdout)
            if res['seconds'] >= 0.3 * target_s or n >= len(qs):
                break
            n = min(len(qs), int(n * max(2.0, target_s / max(res['seconds'], 1e-3))))
    return res


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
        try:
            self.f = open(self.path, 'w')
            self.proc = subprocess.Popen(['nvidia-smi', '--query-gpu=' + q, '--format=csv',
                                          '-lms', '200'], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self, device_index):
        try:
            rows = [l.strip().split(', ') for l in open(self.path).read().strip().splitlines()[1:]]
        except OSError:
            return None
        rows = [r for r in rows if len(r) >= 9 and r[0] == str(device_index)]
        if not rows:
            return None
        mhz = [float(r[1].split()[0]) for r in rows]
        mx = float(rows[0][2].split()[0])
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == 'Active'})
        return {'sm_mhz': statistics.median(mhz), 'sm_max_mhz': mx, 'reasons': reasons,
                'samples': len(rows)}


def run_reference(args, rank, world):
    from libcint_gb300 import molecules as M
    if rank != 0:
        return
    mol = M.config1(seed=0)
    qs = load_quartets(args.quartets)
    threads = os.cpu_count()
    rates = []
    for step in range(args.warmup + args.steps):
        res = cpu_port_rate(mol, qs, threads, target_s=args.cpu_seconds)
        if step >= args.warmup:
            rates.append(res['integrals'] / res['seconds'])
    v = float(np.median(rates))
    line = {
        'impl': 'reference', 'metric': METRIC,
        'value': v, 'unit': 'integrals/s', 'n_gpus': args.gpus, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': 1e3 * res['seconds'], 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
        'config': {'workload': 'c1: 120 atoms, 14 A cube, 3s3p2d1f, 1-8 prims, Schwarz 1e-12',
                   'quartets_per_step': res['quartets']},
        'cpu_baseline': {'value': v, 'unit': 'integrals/s', 'cores': res['threads'], 'kind': 'port',
                         'sample': '%d Schwarz-surviving c1 quartets, OpenMP dynamic, table roots'
                                   % res['quartets']},
        'e2e': {'value': v, 'unit': 'integrals/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'note': 'libcint itself is not buildable on the GPU host (its sources are not shipped); '
                'the timed CPU implementation is the C restatement in oracle/ with table roots '
                '(same checksum as libcint on a shared sample; about 7x slower than libcint on '
                'the same cores in the build container).',
    }
    print(json.dumps(line), flush=True)


def _timed(fn, reps=3):
    import torch
    fn()
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best


def extra_dropin(cg, mol, qs, batched_value, n=4000):
    """The plain drop-in on its own workload, c0 (8 atoms, 6 A, s,s,p,p,d x 4
    primitives): one libcint-signature int2e_sph call per quartet from host buffers, without and
    with an int2e_optimizer (whose side table caches the shell pairs' primitive data), on the first
    n of its 336,610 unique quartets, from one host thread and from 4, 16 and all host threads at
    once (libcint's OpenMP caller pattern); and the batched plan over the whole c0 list for the
    ratio."""
    import torch
    from libcint_gb300 import molecules as M
    m0 = M.config0(seed=0)
    allq = M.unique_quartets(m0.nbas)
    sub = allq[:n]
    nint = integrals_of(m0, sub)
    buf = np.zeros(int(max(np.prod([m0.nsph(s) for s in q]) for q in sub)))
    L = cg.lib()
    f = L.int2e_sph
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    opt = ctypes.c_void_p()
    L.int2e_optimizer(ctypes.byref(opt), P(m0.atm), m0.natm, P(m0.bas), m0.nbas, P(m0.env))
    res = {'workload': 'c0 (8 atoms, 6 A, s,s,p,p,d x 4 prims): first %d of its %d unique quartets, '
                       'one int2e_sph call each' % (n, len(allq))}
    for tag, o in (('no_optimizer', None), ('with_optimizer', opt)):
        f(P(buf), None, P(np.ascontiguousarray(sub[0])), P(m0.atm), m0.natm, P(m0.bas), m0.nbas,
          P(m0.env), o, None)
        t0 = time.perf_counter()
        for q in sub:
            f(P(buf), None, P(np.ascontiguousarray(q)), P(m0.atm), m0.natm, P(m0.bas), m0.nbas,
              P(m0.env), o, None)
        dt = time.perf_counter() - t0
        res[tag] = {'integrals_per_s': nint / dt, 'quartets_per_s': n / dt}
    # libcint's caller pattern: host threads calling int2e_sph concurrently (each thread its own
    # output buffer, one shared optimizer; the library keeps a stream per thread)
    import threading
    rows = [np.ascontiguousarray(q) for q in sub]
    args = (P(m0.atm), m0.natm, P(m0.bas), m0.nbas, P(m0.env), opt, None)
    res['threads'] = {}
    for nth in sorted({4, 16, os.cpu_count() or 16}):
        bufs = [np.zeros_like(buf) for _ in range(nth)]

        def work(t):
            b = P(bufs[t])
            for i in range(t, len(rows), nth):
                f(b, None, P(rows[i]), *args)
        th = [threading.Thread(target=work, args=(t,)) for t in range(nth)]
        t0 = time.perf_counter()
        for x in th:
            x.start()
        for x in th:
            x.join()
        dt = time.perf_counter() - t0
        res['threads'][str(nth)] = {'integrals_per_s': nint / dt, 'quartets_per_s': n / dt}
    L.CINTdel_optimizer(ctypes.byref(opt))
    p = cg.Plan(cg.INT2E_SPH, m0, allq)
    out = torch.empty(p.output_size, dtype=torch.float64, device='cuda')
    dtb = _timed(lambda: p.execute(out))
    p.close()
    vb = integrals_of(m0, allq) / dtb
    res['batched_whole_c0_integrals_per_s'] = vb
    res['batched_over_dropin'] = vb / res['no_optimizer']['integrals_per_s']
    res['batched_over_dropin_with_optimizer'] = vb / res['with_optimizer']['integrals_per_s']
    return res


def extra_int3c2e(cg, seed=0, npairs=40):
    """c2: (ij|P) for screened orbital pairs against every auxiliary shell, batched."""
    import torch
    from libcint_gb300 import molecules as M
    mol, norb = M.config2(seed=seed)
    # unit zero-exponent s shell for (P|P) = (P fit|P fit) (libcint testsuite/test_3c2e.py:134-146)
    env = list(mol.env)
    pe = len(env)
    env += [0.0, 2.0 * np.sqrt(np.pi)]
    bas = np.vstack([mol.bas, [[0, 0, 1, 1, 0, pe, pe + 1, 0]]]).astype(np.int32)
    molf = M.Mol(mol.atm, bas, np.array(env), mol.name)
    fit = bas.shape[0] - 1
    aux = np.arange(norb, mol.nbas, dtype=np.int32)

    def diag_max(items):
        p = cg.Plan(cg.INT2E_SPH, molf, items)
        out = torch.zeros(p.output_size, dtype=torch.float64, device='cuda')
        p.execute(out)
        torch.cuda.synchronize()
        v = np.abs(out.cpu().numpy())
        d = np.array([molf.nsph(int(a)) * molf.nsph(int(b)) for a, b, _, _ in items]) ** 2
        return np.maximum.reduceat(v, np.concatenate([[0], np.cumsum(d)[:-1]]))
    qp = np.sqrt(diag_max(np.stack([aux, np.full_like(aux, fit), aux, np.full_like(aux, fit)], 1)))
    rng = np.random.RandomState(seed)
    ii = rng.randint(0, norb, 4 * npairs)
    jj = rng.randint(0, norb, 4 * npairs)
    pr = np.unique(np.stack([np.maximum(ii, jj), np.minimum(ii, jj)], 1), axis=0)[:npairs * 2]
    qij = np.sqrt(diag_max(np.concatenate([pr, pr], 1).astype(np.int32)))
    keep = qij * qp.max() >= 1e-12
    pr = pr[keep][:npairs]
    qij = qij[keep][:npairs]
    tri = np.array([(i, j, P) for (i, j), q in zip(pr, qij) for P, qq in zip(aux, qp)
                    if q * qq >= 1e-12], dtype=np.int32)
    p = cg.Plan(cg.INT3C2E_SPH, mol, tri)
    out = torch.empty(p.output_size, dtype=torch.float64, device='cuda')
    dt = _timed(lambda: p.execute(out))
    nint = sum(mol.nsph(int(a)) * mol.nsph(int(b)) * mol.nsph(int(c)) for a, b, c in tri)
    # int2c2e: the metric (P|Q) over every unique pair of auxiliary shells (P >= Q)
    pi, qi = np.tril_indices(len(aux))
    pq = np.stack([aux[pi], aux[qi]], 1).astype(np.int32)
    p2 = cg.Plan(cg.INT2C2E_SPH, mol, pq)
    out2 = torch.empty(p2.output_size, dtype=torch.float64, device='cuda')
    dt2 = _timed(lambda: p2.execute(out2))
    ns = np.array([mol.nsph(int(a)) for a in aux], dtype=np.int64)
    nint2 = int((ns[pi] * ns[qi]).sum())
    return {'workload': 'c2: 200 atoms, 18 A; %d screened orbital pairs x all 2000 aux shells '
                        '(Q_ij Q_P >= 1e-12)' % len(pr),
            'triples': int(len(tri)), 'integrals_per_s': nint / dt, 'ms': 1e3 * dt,
            'fp64_frac': p.flops / dt / 1e12 / FP64_PEAK_TFLOPS,
            'int2c2e_metric': {'pairs': int(len(pq)), 'integrals': nint2, 'ms': 1e3 * dt2,
                               'integrals_per_s': nint2 / dt2}}


def planning_threads():
    """host threads that plan chunks ahead of the GPU: all cores but two, at most 12 (each holds
    one chunk plan, ~1 GB of host memory at 4M triples)"""
    return max(1, min(12, (os.cpu_count() or 8) - 2))


def extra_c2(cg, seed=0, thr=1e-12, chunk=4_000_000):
    """c2 at full size: the whole Schwarz-screened (ij|P) tensor (Q_ij Q_P >= 1e-12 over every
    orbital shell pair i >= j and every auxiliary shell), evaluated in streamed chunks of about
    4M triples (planned on host threads ahead of the GPU, each run into one reused device buffer;
    nothing is kept).  Reports the triple and integral counts, the bounds' time, the
    planning (summed over threads), device and wall times, and integrals/s on the device and
    overall."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.screening import pair_bounds
    mol, norb = M.config2(seed=seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ii, jj = np.tril_indices(norb)
    pairs = np.stack([ii, jj], 1)
    qij = pair_bounds(mol, pairs)
    # (P|P) of the auxiliary shells as (P s0|P s0) with the unit zero-exponent s shell
    env = list(mol.env)
    pe = len(env)
    env += [0.0, 2.0 * np.sqrt(np.pi)]
    bas = np.vstack([mol.bas, [[0, 0, 1, 1, 0, pe, pe + 1, 0]]]).astype(np.int32)
    molf = M.Mol(mol.atm, bas, np.array(env), mol.name)
    aux = np.arange(norb, mol.nbas, dtype=np.int64)
    fit = np.full_like(aux, bas.shape[0] - 1)
    qp = pair_bounds(molf, np.stack([aux, fit], 1))
    torch.cuda.synchronize()
    t_bounds = time.perf_counter() - t0
    order = np.argsort(-qp, kind='stable')
    qps = qp[order]
    # per pair, the auxiliary shells with Q_ij Q_P >= thr are a prefix of the sorted list
    with np.errstate(divide='ignore'):
        need = np.where(qij > 0, thr / np.where(qij > 0, qij, 1.0), np.inf)
    cnt = np.searchsorted(-qps, -need, side='right')
    keep = cnt > 0
    pairs, cnt = pairs[keep], cnt[keep]
    total = int(cnt.sum())
    L = mol.bas[:, M.ANG_OF]
    ns = (2 * L + 1) * mol.bas[:, M.NCTR_OF]
    # chunks of about `chunk` triples, planned on host threads (ctypes releases the GIL) while
    # the GPU runs earlier chunks; each chunk runs into one reused device buffer
    cum = np.concatenate([[0], np.cumsum(cnt)])
    bounds = []
    a = 0
    while a < len(pairs):
        b = max(int(np.searchsorted(cum, cum[a] + chunk, side='right')) - 1, a + 1)
        bounds.append((a, b))
        a = b

    def triples(a, b):
        c = cnt[a:b]
        tri = np.empty((int(c.sum()), 3), dtype=np.int32)
        tri[:, :2] = np.repeat(pairs[a:b], c, axis=0)
        starts = np.repeat(np.cumsum(c) - c, c)
        tri[:, 2] = aux[order[np.arange(len(tri)) - starts]]
        return tri

    def build(ab):
        tri = triples(*ab)
        t1 = time.perf_counter()
        p = cg.Plan(cg.INT3C2E_SPH, mol, tri)
        return p, time.perf_counter() - t1, int((ns[tri[:, 0]] * ns[tri[:, 1]] * ns[tri[:, 2]]).sum())
    from concurrent.futures import ThreadPoolExecutor
    nint_total, buf, plan_s, dev_s = 0, None, 0.0, 0.0
    torch.cuda.synchronize()
    t_all = time.perf_counter()
    nth = planning_threads()
    with ThreadPoolExecutor(nth) as pool:
        futs = [pool.submit(build, ab) for ab in bounds[:nth]]
        for i in range(len(bounds)):
            p, ps, ni = futs[i].result()
            if i + nth < len(bounds):
                futs.append(pool.submit(build, bounds[i + nth]))
            plan_s += ps
            nint_total += ni
            if buf is None or buf.numel() < p.output_size:
                buf = torch.empty(int(p.output_size * 1.2), dtype=torch.float64, device='cuda')
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            p.execute(buf)
            e1.record()
            e1.synchronize()
            dev_s += e0.elapsed_time(e1) / 1e3
            p.close()
    wall = time.perf_counter() - t_all
    return {'workload': 'c2: 200 atoms, 18 A; every orbital shell pair x every auxiliary shell '
                        'with Q_ij Q_P >= 1e-12', 'orbital_pairs_kept': int(len(pairs)),
            'triples': total, 'integrals': nint_total, 'bounds_s': t_bounds, 'chunks': len(bounds),
            'plan_s_summed_over_threads': plan_s, 'device_s': dev_s, 'wall_s': wall,
            'integrals_per_s_device': nint_total / dev_s, 'integrals_per_s_overall': nint_total / wall}


def extra_adjoint(cg, seed=0, natm=24):
    """c3: 24 atoms (fewer, in a box of the same density, for profiling), full unique quartet
    list; adjoint gradient vs int2e_ip1 formed and contracted on the same GPU; agreement between
    the two."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.coulomb import CoulombPlans, IP1Gradient
    mol = M.config3(seed=seed, natm=natm, box=8.0 * (natm / 24.0) ** (1.0 / 3.0))
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    rng = np.random.RandomState(seed)
    d = rng.normal(0, 0.1, (nao, nao))
    dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    plans = CoulombPlans(mol)
    t_fwd = _timed(lambda: plans.energy(dm))
    g_adj = [None]

    def adj():
        g_adj[0] = plans.grad(dm)[0]
    t_adj = _timed(adj, reps=2)   # the adjoint plan is built by the untimed first call
    # the comparator's three int2e_ip1 plans are built here, outside the timed region, as the
    # adjoint's is: both sides time device work (plus the comparator's contraction)
    route = IP1Gradient(mol)
    g_ip1 = [None]

    def ip1():
        g_ip1[0] = route.grad(dm)
    t_ip1 = _timed(ip1, reps=2)
    route.close()
    diff = float((g_adj[0] - g_ip1[0]).abs().max() / g_ip1[0].abs().max())
    plans_a = CoulombPlans(mol, with_exponents=True)
    t_adj_a = _timed(lambda: plans_a.grad(dm), reps=1)
    return {'workload': 'c3: %d atoms, %.1f A, s,p,d x 3-5 prims, all %d unique quartets'
                        % (natm, 8.0 * (natm / 24.0) ** (1.0 / 3.0), len(M.unique_quartets(mol.nbas))),
            'forward_J_ms': 1e3 * t_fwd, 'adjoint_grad_ms': 1e3 * t_adj,
            'adjoint_grad_with_exponents_ms': 1e3 * t_adj_a, 'ip1_route_grad_ms': 1e3 * t_ip1,
            'adjoint_speedup_over_ip1': t_ip1 / t_adj, 'max_rel_diff_vs_ip1': diff,
            'comparator': 'int2e_ip1 route (three batched plans, built outside the timed region) '
                          'formed in HBM and contracted with torch'}


def extra_jk(cg, seed=0, natm=24):
    """c3 J/K build (the contraction a direct-SCF driver makes of each unique quartet): J alone,
    K alone, and J and K from one evaluation of each quartet; the JK plan's J against the J
    plan's, and K's symmetry."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.coulomb import CoulombPlans
    box = 8.0 * (natm / 24.0) ** (1.0 / 3.0)
    mol = M.config3(seed=seed, natm=natm, box=box)
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    rng = np.random.RandomState(seed)
    d = rng.normal(0, 0.1, (nao, nao))
    dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    plans = CoulombPlans(mol)
    t_j = _timed(lambda: plans.vj(dm), reps=2)
    t_k = _timed(lambda: plans.vk(dm), reps=2)
    res = [None]

    def jk():
        res[0] = plans.get_jk(dm)
    t_jk = _timed(jk, reps=2)
    J, K = res[0]
    J1 = plans.vj(dm)
    return {'workload': 'c3: %d atoms, %.1f A, s,p,d x 3-5 prims, all %d unique quartets'
                        % (natm, box, len(M.unique_quartets(mol.nbas))),
            'J_ms': 1e3 * t_j, 'K_ms': 1e3 * t_k, 'JK_ms': 1e3 * t_jk, 'JK_over_J': t_jk / t_j,
            'jk_J_vs_J_max_rel': float((J - J1).abs().max() / J1.abs().max()),
            'K_asymmetry_max_rel': float((K - K.T).abs().max() / K.abs().max()),
            'coulomb_energy': float(0.5 * (dm * J).sum()), 'exchange_energy': float(-0.25 * (dm * K).sum())}


def hbm_peak_gbs():
    """(GB/s, source): the measured copy bandwidth in MEASURED_PEAKS.json when that file is
    present, else the fallback figure of an earlier GB300 measurement"""
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            v = float(json.load(f)['hbm_gbs'])
        return v, 'measured (MEASURED_PEAKS.json hbm_gbs)'
    except Exception:
        return 6800.0, 'fallback 6.8 TB/s (no MEASURED_PEAKS.json)'


def _df_kernel_times(fit, dm, reps=5):
    """best-of-reps CUDA-event times (ms) of the two DF kernels and of a whole J build"""
    import torch
    c = fit.coefficients(dm)
    out = {}
    for tag, fn in (('rho', lambda: fit.rho(dm)), ('j', lambda: fit.vj_from_coefficients(c)),
                    ('vj', lambda: fit.vj(dm))):
        fn()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            best = e0.elapsed_time(e1) if best is None else min(best, e0.elapsed_time(e1))
        out[tag + '_ms'] = best
    # one FP64 FMA per 8-byte element: the FP64 pipe (measured DFMA peak) streams at most
    # FP64_PEAK_TFLOPS / 2 G elements/s, below HBM, so it is the bound; HBM is reported beside it
    peak, src = hbm_peak_gbs()
    fma_gbs = FP64_PEAK_TFLOPS * 1e12 / 2 * 8 / 1e9
    nbytes = 8.0 * fit.T.numel()
    for tag in ('rho', 'j'):
        gbs = nbytes / (out[tag + '_ms'] * 1e-3) / 1e9
        out[tag + '_roofline'] = {'bound': 'fp64', 'achieved': gbs, 'peak': fma_gbs, 'unit': 'GB/s',
                                  'frac': gbs / fma_gbs, 'algorithmic_bytes': nbytes,
                                  'peak_source': 'one FMA per element at the measured DFMA peak',
                                  'hbm_peak': peak, 'hbm_frac': gbs / peak, 'hbm_peak_source': src}
    return out


def extra_df(cg, seed=0, natm=20):
    """Density-fitted J on a c2-type system (orbital s,s,p,p,d with 1-6 primitives, auxiliary
    l <= 4 x 2 per atom, same density of atoms as c2): set-up (the int3c2e buffer, the metric and
    its Cholesky factor) and one J build, with the two DF kernels' own times against HBM."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.df import DFCoulomb
    box = 18.0 * (natm / 200.0) ** (1.0 / 3.0)
    mol, norb = M.config2(seed=seed, natm=natm, box=box)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fit = DFCoulomb(mol, norb)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    rng = np.random.RandomState(seed)
    d = rng.normal(0, 0.1, (fit.nao, fit.nao))
    dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    t_j = _timed(lambda: fit.vj(dm))
    res = {'workload': 'c2-type: %d atoms, %.1f A, all %d orbital shell pairs x %d aux shells'
                       % (natm, box, norb * (norb + 1) // 2, mol.nbas - norb),
           'nao': fit.nao, 'naux': fit.naux, 'three_index_elements': int(fit.T.numel()),
           'setup_s': t_setup, 'vj_ms': 1e3 * t_j, 'kernels': _df_kernel_times(fit, dm)}
    fit.close()
    return res


def extra_dfc2(cg, seed=0, thr=1e-12):
    """Density-fitted J at c2's full size: 200 atoms, 1000 orbital shells (2600 AOs), 2000
    auxiliary shells (10,000 functions); every orbital shell pair with Q_ij max_P Q_P >= 1e-12
    (the pairs with any surviving triple) x every auxiliary shell, the three-index buffer resident
    in HBM.  Reports the set-up and the J build's kernels against HBM."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.df import DFCoulomb
    from libcint_gb300.screening import pair_bounds
    mol, norb = M.config2(seed=seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ii, jj = np.tril_indices(norb)
    pairs = np.stack([ii, jj], 1)
    qij = pair_bounds(mol, pairs)
    env = list(mol.env)
    pe = len(env)
    env += [0.0, 2.0 * np.sqrt(np.pi)]
    bas = np.vstack([mol.bas, [[0, 0, 1, 1, 0, pe, pe + 1, 0]]]).astype(np.int32)
    molf = M.Mol(mol.atm, bas, np.array(env), mol.name)
    aux = np.arange(norb, mol.nbas, dtype=np.int64)
    qp = pair_bounds(molf, np.stack([aux, np.full_like(aux, bas.shape[0] - 1)], 1))
    keep = qij * qp.max() >= thr
    t_bounds = time.perf_counter() - t0
    t0 = time.perf_counter()
    fit = DFCoulomb(mol, norb, pairs=pairs[keep])
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    rng = np.random.RandomState(seed)
    d = torch.as_tensor(rng.normal(0, 0.1, (fit.nao, fit.nao)), device='cuda')
    dm = 0.5 * (d + d.T)
    res = {'workload': 'c2 full: 200 atoms, 18 A; %d of %d orbital shell pairs (Q_ij max Q_P >= 1e-12) '
                       'x all %d auxiliary shells' % (int(keep.sum()), len(pairs), len(aux)),
           'nao': fit.nao, 'naux': fit.naux, 'three_index_elements': int(fit.T.numel()),
           'three_index_gb': 8e-9 * fit.T.numel(), 'bounds_s': t_bounds, 'setup_s': t_setup,
           'kernels': _df_kernel_times(fit, dm, reps=3)}
    fit.close()
    return res


def extra_screening(cg, seed=0, natm=24, threshold=1e-10):
    """c3 J/K with Schwarz/density screening against the full unique list: Schwarz bounds (one
    int2e_sph plan over the diagonal quartets), the screened plan's size and time, and the largest
    change of J and K."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.coulomb import CoulombPlans
    from libcint_gb300.screening import schwarz_bounds, screened_coulomb_plans
    box = 8.0 * (natm / 24.0) ** (1.0 / 3.0)
    mol = M.config3(seed=seed, natm=natm, box=box)
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    rng = np.random.RandomState(seed)
    d = rng.normal(0, 0.1, (nao, nao))
    dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    full = CoulombPlans(mol)
    res = [None]

    def jk_full():
        res[0] = full.get_jk(dm)
    t_full = _timed(jk_full, reps=2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Q = schwarz_bounds(mol)
    t_q = time.perf_counter() - t0
    t0 = time.perf_counter()
    sp = screened_coulomb_plans(mol, dm, threshold, Q)
    t_plan = time.perf_counter() - t0
    res2 = [None]

    def jk_scr():
        res2[0] = sp.get_jk(dm)
    t_scr = _timed(jk_scr, reps=2)
    (J0, K0), (J1, K1) = res[0], res2[0]
    return {'workload': 'c3: %d atoms, %.1f A, random symmetric density, threshold %g' % (natm, box, threshold),
            'quartets': int(len(full.quartets)), 'kept': int(len(sp.quartets)),
            'jk_ms': 1e3 * t_full, 'screened_jk_ms': 1e3 * t_scr, 'schwarz_ms': 1e3 * t_q,
            'screened_plan_s': t_plan,
            'max_abs_dJ': float((J1 - J0).abs().max()), 'max_abs_dK': float((K1 - K0).abs().max())}


def _screened_total(q, threshold):
    """quartets of the whole Schwarz-screened unique list (ScreenedCoulomb's enumeration) and the
    per-bra-position counts, from the pair bounds alone"""
    qs = np.sort(np.asarray(q))[::-1]
    pos = np.arange(len(qs))
    with np.errstate(divide='ignore'):
        need = np.where(qs > 0, threshold / np.where(qs > 0, qs, 1.0), np.inf)
    # kets of position p: pairs with bound >= need, at most p + 1
    n = len(qs) - np.searchsorted(qs[::-1], need, side='left')
    k = np.where(qs > 0, np.minimum(pos + 1, n), 0)
    return int(k.sum()), k


def _slab_range(k, nq):
    """bra positions [p0, p1) that enumerate about nq quartets, starting where half of the whole
    list has been enumerated (the median quartet, not the median pair: most distant pairs have
    few partners)"""
    cum = np.cumsum(k)
    p0 = int(np.searchsorted(cum, cum[-1] / 2))
    p1 = int(np.searchsorted(cum, cum[p0] - k[p0] + nq)) + 1
    return p0, max(p0 + 1, min(p1, len(k)))


def extra_screened(cg, natm_whole=12, slab_quartets=4.0e6, seed=0):
    """Whole-molecule Schwarz-screened J (c1, Q_ij Q_kl >= 1e-12) through
    cintgpu_screened_run, which never stores the quartet list: the bounds of all 583k c1 shell
    pairs, a timed slab of bra pairs from the median quartet on (extrapolated to the whole list by
    quartet count), and a whole c1-density molecule of natm_whole atoms timed end to end."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.screening import ScreenedCoulomb
    out = {}
    for tag, mol in (('c1', M.config1(seed=seed)),
                     ('whole', M.config1(seed=seed, natm=natm_whole,
                                         box=14.0 * (natm_whole / 120.0) ** (1.0 / 3.0)))):
        nao = sum(mol.nsph(i) for i in range(mol.nbas))
        d = np.random.RandomState(seed).normal(0, 0.1, (nao, nao))
        dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc = ScreenedCoulomb(mol, threshold=SCHWARZ)
        torch.cuda.synchronize()
        t_q = time.perf_counter() - t0
        total, k = _screened_total(sc.q, SCHWARZ)
        if tag == 'c1':
            rng_ = _slab_range(k, slab_quartets)
        else:
            rng_ = None
        sc.get_jk(dm, True, False, bra_range=rng_ if rng_ else (0, min(len(k), 64)))   # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc.get_jk(dm, True, False, bra_range=rng_)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        nq = sc.last_quartets
        r = {'atoms': mol.natm, 'shell_pairs': int(len(sc.pairs)), 'bounds_s': t_q,
             'surviving_quartets': total, 'unique_quartets': int(len(sc.pairs) * (len(sc.pairs) + 1) // 2),
             'timed_quartets': nq, 'J_s': dt, 'quartets_per_s': nq / dt}
        if tag == 'c1':
            r['slab'] = 'bra positions [%d, %d) of %d in bound order' % (rng_[0], rng_[1], len(k))
            r['extrapolated_whole_J_s'] = dt * total / max(nq, 1)
        out[tag] = r
    return out


def _slab_list(sc, p0, p1):
    """the quartets ScreenedCoulomb evaluates for bra positions [p0, p1), materialised"""
    order = np.argsort(-sc.q, kind='stable')
    qs = sc.q[order]
    out = []
    for p in range(p0, p1):
        if qs[p] <= 0:
            continue
        k = int(np.count_nonzero(qs[:p + 1] * qs[p] >= SCHWARZ))
        bra = np.broadcast_to(sc.pairs[order[p]], (k, 2))
        out.append(np.concatenate([bra, sc.pairs[order[:k]]], 1))
    return np.ascontiguousarray(np.concatenate(out), dtype=np.int32)


def extra_c4(cg, seed=0, slab_j=1.5e6, slab_grad=1.5e5):
    """c4 at full size (400 atoms, 24 A, s:3 p:3 d:2 f:1 g:1, 1-8 primitives, 4000 shells, 8M
    shell pairs), Schwarz 1e-12: the bounds of every pair, the whole surviving list's size, a
    timed J slab and a timed adjoint slab (bra pairs from the median quartet on; the list is
    streamed, never stored), and the adjoint against forming int2e_ip1 and contracting it on the
    head of the adjoint slab's list (both planned outside the timed region) with the two
    gradients' agreement."""
    import torch
    from libcint_gb300 import molecules as M
    from libcint_gb300.coulomb import IP1Gradient
    from libcint_gb300.screening import ScreenedCoulomb
    mol = M.config4(seed=seed)
    nao = sum(mol.nsph(i) for i in range(mol.nbas))
    d = np.random.RandomState(seed).normal(0, 0.1, (nao, nao))
    dm = torch.as_tensor(0.5 * (d + d.T), device='cuda')
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sc = ScreenedCoulomb(mol, threshold=SCHWARZ)
    torch.cuda.synchronize()
    t_q = time.perf_counter() - t0
    total, k = _screened_total(sc.q, SCHWARZ)
    pj = _slab_range(k, slab_j)
    pg = _slab_range(k, slab_grad)
    mid = pj[0]
    res = {'workload': 'c4: 400 atoms, 24 A, 3s3p2d1f1g, 1-8 prims, Schwarz 1e-12',
           'shell_pairs': int(len(sc.pairs)), 'bounds_s': t_q, 'surviving_quartets': total}
    from libcint_gb300.coulomb import J_BUILD, J_GRAD
    dmc = sc.dm_cart(dm)          # the streamed contraction alone is timed
    XJ = torch.zeros_like(dmc)
    sc._run(J_BUILD, dmc, vj=XJ, bra_range=(mid, mid + 2))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sc._run(J_BUILD, dmc, vj=XJ, bra_range=pj)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    res['J_slab'] = {'quartets': sc.last_quartets, 's': dt, 'quartets_per_s': sc.last_quartets / dt,
                     'extrapolated_whole_s': dt * total / max(sc.last_quartets, 1)}
    g = torch.zeros((mol.natm, 3), dtype=torch.float64, device='cuda')
    sc._run(J_GRAD, dmc, g=g, bra_range=(mid, mid + 2))
    g.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sc._run(J_GRAD, dmc, g=g, bra_range=pg)
    torch.cuda.synchronize()
    dg = time.perf_counter() - t0
    nq = sc.last_quartets
    res['adjoint_slab'] = {'quartets': nq, 'adjoint_s': dg, 'quartets_per_s': nq / dg,
                           'extrapolated_whole_adjoint_s': dg * total / max(nq, 1),
                           'note': 'streamed: includes the chunk planning on host threads'}
    # like for like against forming int2e_ip1 and contracting, on the head of the adjoint slab's
    # list: the comparator stores 3 spherical derivative blocks per quartet (up to 15^4 doubles
    # each for (gg|gg)), so the list is cut where those reach 8 GB
    try:
        from libcint_gb300.coulomb import CoulombPlans
        lst = _slab_list(sc, *pg)
        L = mol.bas[:, M.ANG_OF]
        nsph = (2 * L + 1) * mol.bas[:, M.NCTR_OF]
        nbytes = np.cumsum(24.0 * np.prod(nsph[lst].astype(np.float64), axis=1))
        sub = lst[:max(1, int(np.searchsorted(nbytes, 8e9)))]
        plans = CoulombPlans(mol, sub)
        plans.grad(dm)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ga = plans.grad(dm)[0]
        torch.cuda.synchronize()
        da = time.perf_counter() - t0
        route = IP1Gradient(mol, sub)
        route.grad(dm)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g1 = route.grad(dm)
        torch.cuda.synchronize()
        di = time.perf_counter() - t0
        route.close()
        res['adjoint_vs_ip1'] = {'quartets': int(len(sub)), 'adjoint_s': da, 'ip1_route_s': di,
                                 'adjoint_speedup_over_ip1': di / da,
                                 'max_rel_diff_vs_ip1': float((ga - g1).abs().max() / g1.abs().max()),
                                 'note': 'both from plans built outside the timed region'}
    except Exception as e:  # the slab numbers above stand without the comparator
        res['adjoint_vs_ip1'] = {'error': repr(e)[:300]}
    return res


def extra_fp64peak():
    """Issue-rate peaks of this GPU (bench_fp64_peak.cu): DFMA, DMMA (FP64 tensor cores) and FFMA
    in TFLOP/s, the best launch shape of each."""
    src = os.path.join(ROOT, 'bench_fp64_peak.cu')
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, 'fp64_peak')
        subprocess.run(['nvcc', '-gencode', 'arch=compute_103a,code=sm_103a', '-O3', '-o', exe, src],
                       check=True)
        r = subprocess.run([exe], capture_output=True, text=True, check=True)
    best, lanes = {}, {}
    for line in r.stdout.splitlines():
        parts = line.split()
        if parts and parts[0] in ('DFMA', 'DMMA', 'FFMA') and line.endswith('TFLOP/s'):
            v = float(parts[-2])
            best[parts[0]] = max(best.get(parts[0], 0.0), v)
        elif parts and parts[0] == 'DFMA-lanes':
            lanes[parts[1].split('=')[1]] = float(parts[parts.index('G') - 1])
    return {'tflops': best, 'dmma_over_dfma': best.get('DMMA', 0) / max(best.get('DFMA', 1e-9), 1e-9),
            'dfma_warp_instr_per_s_by_active_lanes': lanes,
            'raw': r.stdout.strip().splitlines()}


def run_extras(cg, mol, qs, value, args):
    out = {}
    for name, fn in (('fp64peak', lambda: {k: v for k, v in extra_fp64peak().items() if k != 'raw'}),
                     ('dropin', lambda: extra_dropin(cg, mol, qs, value)),
                     ('int3c2e', lambda: extra_int3c2e(cg)),
                     ('adjoint', lambda: extra_adjoint(cg)),
                     ('jk', lambda: extra_jk(cg)),
                     ('screening', lambda: extra_screening(cg)),
                     ('df', lambda: extra_df(cg)),
                     ('c2', lambda: extra_c2(cg)),
                     ('dfc2', lambda: extra_dfc2(cg))):
        try:
            out[name] = fn()
        except Exception as e:  # an extra must not hide the headline line
            out[name] = {'error': repr(e)[:300]}
    return out


def run_gpu(args, rank, world):
    import torch
    import libcint_gb300 as cg
    from libcint_gb300 import molecules as M
    dev = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(dev)
    cg.build_library()
    if args.only != 'headline':
        # one side workload alone (profiling); not the benchmark line
        fn = {'adjoint': lambda: extra_adjoint(cg, natm=args.c3_atoms),
              'jk': lambda: extra_jk(cg, natm=args.c3_atoms),
              'df': lambda: extra_df(cg),
              'screening': lambda: extra_screening(cg, natm=args.c3_atoms),
              'int3c2e': lambda: extra_int3c2e(cg),
              'fp64peak': extra_fp64peak,
              'screened': lambda: extra_screened(cg),
              'c4': lambda: extra_c4(cg),
              'c2': lambda: extra_c2(cg),
              'dropin': lambda: extra_dropin(cg, None, None, None),
              'dfc2': lambda: extra_dfc2(cg)}[args.only]
        if rank == 0:
            print(json.dumps({'extra': args.only, **fn()}), flush=True)
        return
    mol = M.config1(seed=0)
    qs = load_quartets(args.quartets)
    nint = integrals_of(mol, qs)
    tuning = None
    if args.tune:
        # launch parameters picked by the autotuner on this list, before any timing
        from libcint_gb300 import autotune
        choice, times = autotune.tune(cg.INT2E_SPH, mol, qs)
        wide, class_ms = autotune.tune_classes(cg.INT2E_SPH, mol, qs, *choice)
        tuning = {'choice': {'ws_kb': choice[0], 'separate_output': choice[1], 'wide_classes': list(wide)},
                  'candidate_ms': {'%d,%d' % c: round(t, 3) for c, t in times.items()},
                  'class_whole_list_ms_regular_wide': {str(k): [round(a, 3), round(b, 3)]
                                                       for k, (a, b) in class_ms.items()}}
        plan = cg.Plan(cg.INT2E_SPH, mol, qs, ws_kb=choice[0], separate_output=choice[1],
                       wide_classes=wide)
    else:
        plan = cg.Plan(cg.INT2E_SPH, mol, qs)
    out = torch.empty(plan.output_size, dtype=torch.float64, device='cuda')
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device='cuda')
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        plan.execute(out, stream)
    torch.cuda.synchronize()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    clk = ClockSampler(os.path.join(os.environ.get('BENCH_CLOCKS_DIR', tempfile.gettempdir()),
                                    'cintgpu_clocks_rank%d.csv' % rank))
    evs = []
    kernel_ms = []
    with clk:
        time.sleep(0.3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.execute(out, stream)
            e1.record(stream)
            evs.append((e0, e1))
            # the integral kernel alone (events the plan records on the same stream); waits for
            # this step, outside the step's own events
            kernel_ms.append(plan.compute_ms())
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    tot_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([tot_s], device='cuda')
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_s = float(t.item())
    # end-to-end through the one-shot host-buffer C-ABI call
    host_out = np.zeros(plan.output_size)
    e2e_times = []
    for it in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        t1 = time.perf_counter()
        rc = cg.lib().cintgpu_batch_host(cg.INT2E_SPH, host_out.ctypes.data_as(ctypes.c_void_p),
                                         qs.ctypes.data_as(ctypes.c_void_p), len(qs), None,
                                         mol.atm.ctypes.data_as(ctypes.c_void_p), mol.natm,
                                         mol.bas.ctypes.data_as(ctypes.c_void_p), mol.nbas,
                                         mol.env.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise RuntimeError(cg.last_error())
        if it > 0:
            e2e_times.append(time.perf_counter() - t1)
    h2d = int(cg.lib().cintgpu_plan_upload_bytes(plan._h)) + qs.nbytes
    d2h = plan.output_size * 8
    if rank != 0:
        return
    value = nint * world * args.steps / tot_s
    kern_s = sum(kernel_ms) / 1e3
    achieved = plan.flops * args.steps / kern_s / 1e12
    clocks = clk.summary(dev)
    line = {
        'metric': METRIC,
        'value': value, 'unit': 'integrals/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': 1e3 * tot_s / args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
        'config': {'workload': 'c1: 120 atoms, 14 A cube, 3s3p2d1f, 1-8 prims, Schwarz 1e-12',
                   'quartets_per_step': int(len(qs)), 'integrals_per_step': nint,
                   'prim_quartets_per_step': int(plan.prim_quartets),
                   'l2': 'flushed before every step (256 MiB memset), outside the step events',
                   'wall_s_timed_region': wall, 'tuning': tuning},
        'quartets_per_s': len(qs) * world * args.steps / tot_s,
        'gpu_launches': plan.launches * args.steps,
        'roofline': {'bound': 'fp64', 'kernel': 'rys_eri_kernel_e0f0',
                     'kernel_ms_per_launch': 1e3 * kern_s / args.steps,
                     'achieved': achieved, 'peak': FP64_PEAK_TFLOPS,
                     'unit': 'TFLOP/s', 'frac': achieved / FP64_PEAK_TFLOPS,
                     'traffic': ERI_DRAM_BYTES_PER_QUARTET * len(qs),
                     'traffic_source': 'ncu dram__bytes_read+write of the 100k-quartet step '
                                       '(scaled by quartets for other lengths)',
                     'flop_model': 'this implementation: per term 20 + 15 VRR entries (+ the bra '
                                   'transfers of bra-per-term classes) + groups + 2 nE nF (FMA = 2)',
                     'libcint_algorithm_tflops': plan.flops_libcint * args.steps / kern_s / 1e12,
                     'libcint_algorithm_note': "the same quartets counted with libcint's "
                                               'per-primitive VRR + HRR + gout model, over the '
                                               'same kernel time (exceeds the pipe peak by the '
                                               'work contraction-first saves)',
                     'peak_source': 'measured DFMA peak (bench.py --only fp64peak); '
                                    'MEASURED_PEAKS.json carries no FP64 figure'},
        'e2e': {'value': nint / statistics.median(e2e_times) if e2e_times else None,
                'unit': 'integrals/s',
                'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h,
                'path': 'cintgpu_batch_host (plan + H2D + kernels + D2H), wall clock'},
        'clocks': clocks,
    }
    if not args.no_extras:
        line['extras'] = run_extras(cg, mol, qs, value, args)
    if not args.no_cpu:
        res = cpu_port_rate(mol, qs, os.cpu_count(), target_s=args.cpu_seconds)
        line['cpu_baseline'] = {'value': res['integrals'] / res['seconds'], 'unit': 'integrals/s',
                                'cores': res['threads'], 'kind': 'port',
                                'sample': 'first %d quartets of the step list (%.1f s)'
                                          % (res['quartets'], res['seconds'])}
        one = cpu_port_rate(mol, qs, 1, target_s=3.0)
        line['cpu_baseline']['one_thread'] = {'value': one['integrals'] / one['seconds'],
                                              'sample': 'first %d quartets (%.1f s)'
                                                        % (one['quartets'], one['seconds'])}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gpu', choices=['gpu', 'reference'])
    ap.add_argument('--quartets', type=int, default=0, help='0 = the whole committed sample')
    ap.add_argument('--e2e-steps', type=int, default=3)
    ap.add_argument('--cpu-seconds', type=float, default=12.0)
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-tune', dest='tune', action='store_false',
                    help='default launch parameters instead of the autotuner\'s choice')
    ap.add_argument('--no-extras', action='store_true', help='skip the side workloads (drop-in, int3c2e, adjoint, J/K, screening, DF, '
                                                             'c2 at full size)')
    ap.add_argument('--only', default='headline', choices=['headline', 'adjoint', 'int3c2e', 'jk', 'df', 'screening',
                                                          'fp64peak', 'screened', 'c4', 'c2', 'dropin', 'dfc2'],
                    help='run one side workload alone and print its line (profiling)')
    ap.add_argument('--c3-atoms', type=int, default=24, help='atoms of the adjoint workload')
    args = ap.parse_args()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if world > 1:
        import torch.distributed as dist
        backend = 'gloo' if args.impl == 'reference' else 'nccl'
        if backend == 'nccl':
            import torch
            torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
        dist.init_process_group(backend)
    if args.impl == 'reference':
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
