"""Generate the Rys root/weight tables evaluated by the GPU kernels (rys_tables.inc).

Run once, offline (needs mpmath):  python gen_rys_tables.py [--nmax 14] [--out rys_tables.inc]

For every root count n = 1..NMAX the x axis [0, X_n) with X_n = 40 + 5n is cut into intervals of
width H (X_n rounded up to a multiple of H).  On each interval the nodes s_i(x) = t_i^2 and weights w_i(x) of the Rys quadrature
(int_0^1 f(t^2) exp(-x t^2) dt, the contract of libcint's CINTrys_roots,
src/rys_roots.c:57-122) are interpolated at DEG+1 Chebyshev points of the first kind by a degree
DEG polynomial, stored in the monomial basis of y = 2 (x - x0)/H - 1 for Horner evaluation.
Beyond X_n the half-range Gauss-Hermite limit is used: s_i = r_i / x, w_i = W_i / sqrt(x), with
r_i = y_i^2 for the positive nodes y_i of H_{2n}.  X_n keeps that limit below 1e-16 (checked by
the generator).  Values come from rys_exact.py at 60 digits.

Layout written (all doubles as exact hexadecimal literals):
  rys_coef[off_n + ((k * n + i) * (DEG + 1) + j) * 2 + {0: s, 1: w}]   k = interval, i = root,
                                                                        j = power of y
  rys_large_r[n(n-1)/2 + i], rys_large_w[n(n-1)/2 + i]
The oracle never uses these tables: it computes its roots independently.
"""
import argparse
import math
import os
import sys
from multiprocessing import Pool

import mpmath

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import rys_exact as R  # noqa: E402

H = 1.0
DEG = 10


def set_grid(h, deg):
    global H, DEG
    H, DEG = h, deg


def xmax_of(n):
    # 40 + 5n rounded up to a whole number of intervals
    return H * math.ceil((40.0 + 5.0 * n) / H)


def nint_of(n):
    return int(xmax_of(n) / H)


def _interval(args):
    n, k = args
    with mpmath.workdps(R.DPS):
        x0 = mpmath.mpf(k) * H
        npt = DEG + 1
        ys = [mpmath.cos(mpmath.pi * (j + mpmath.mpf(1) / 2) / npt) for j in range(npt)]
        vals = []
        for y in ys:
            x = x0 + (y + 1) * H / 2
            s, w = R.rys_exact(n, x)
            vals.append((s, w))
        out = []
        for i in range(n):
            for which in (0, 1):
                f = [vals[p][which][i] for p in range(npt)]
                # Chebyshev coefficients c_j = (2/npt) sum_p f_p T_j(y_p), c_0 halved
                c = []
                for j in range(npt):
                    acc = mpmath.mpf(0)
                    for p in range(npt):
                        acc += f[p] * mpmath.cos(j * mpmath.acos(ys[p]))
                    c.append(acc * 2 / npt)
                c[0] /= 2
                # Chebyshev -> monomial in y (exact arithmetic at DPS digits)
                mono = [mpmath.mpf(0)] * npt
                tkm1 = [mpmath.mpf(1)] + [mpmath.mpf(0)] * (npt - 1)      # T_0
                tk = [mpmath.mpf(0), mpmath.mpf(1)] + [mpmath.mpf(0)] * (npt - 2)  # T_1
                for j in range(npt):
                    tj = tkm1 if j == 0 else tk if j == 1 else None
                    if j >= 2:
                        tnew = [mpmath.mpf(0)] * npt
                        for a in range(npt - 1):
                            tnew[a + 1] += 2 * tk[a]
                        for a in range(npt):
                            tnew[a] -= tkm1[a]
                        tkm1, tk = tk, tnew
                        tj = tk
                    for a in range(npt):
                        mono[a] += c[j] * tj[a]
                out.append([float(v) for v in mono])
        return n, k, out


def _check_large(n):
    ys, ws = R.hermite_half(n)
    x = xmax_of(n)
    s, w = R.rys_exact(n, x)
    F0 = sum(w)
    es = max(abs(float(a - y * y / x)) for a, y in zip(s, ys))
    ew = max(abs(float((a - W / mpmath.sqrt(x)) / F0)) for a, W in zip(w, ws))
    return n, [float(y * y) for y in ys], [float(W) for W in ws], es, ew


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--nmax', type=int, default=14)
    ap.add_argument('--out', default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                  'rys_tables.inc'))
    ap.add_argument('--procs', type=int, default=os.cpu_count())
    ap.add_argument('--h', type=float, default=H)
    ap.add_argument('--deg', type=int, default=DEG)
    args = ap.parse_args()
    set_grid(args.h, args.deg)
    nmax = args.nmax
    jobs = [(n, k) for n in range(1, nmax + 1) for k in range(nint_of(n))]
    with Pool(args.procs, initializer=set_grid, initargs=(args.h, args.deg)) as pool:
        res = pool.map(_interval, jobs, chunksize=1)
        large = pool.map(_check_large, range(1, nmax + 1))
    table = {}
    for n, k, out in res:
        table[(n, k)] = out
    offs, coef = [], []
    for n in range(1, nmax + 1):
        offs.append(len(coef))
        for k in range(nint_of(n)):
            out = table[(n, k)]
            for i in range(n):
                s_mono, w_mono = out[2 * i], out[2 * i + 1]
                for j in range(DEG + 1):
                    coef.append(s_mono[j])
                    coef.append(w_mono[j])
    lr, lw = [], []
    for n, r, w, es, ew in large:
        if es > 1e-16 or ew > 1e-16:
            raise SystemExit('large-x limit too coarse at n=%d: %g %g' % (n, es, ew))
        lr += r
        lw += w
    with open(args.out, 'w') as f:
        f.write('/* Generated by gen_rys_tables.py -- do not edit.  Rys nodes s=t^2 and weights:\n'
                ' * piecewise degree-%d polynomials on intervals of width %g for x < 40+5n,\n'
                ' * half-range Gauss-Hermite limit beyond.  See the generator for the layout. */\n'
                % (DEG, H))
        f.write('#define RYS_NMAX %d\n#define RYS_DEG %d\n#define RYS_H %.1f\n#define RYS_INV_H %.17g\n'
                % (nmax, DEG, H, 1.0 / H))
        f.write('static const int rys_nint_host[RYS_NMAX + 1] = {0, %s};\n'
                % ', '.join(str(nint_of(n)) for n in range(1, nmax + 1)))
        f.write('static const int rys_off_host[RYS_NMAX + 1] = {0, %s};\n'
                % ', '.join(str(o) for o in offs))
        f.write('#define RYS_NCOEF %d\n' % len(coef))
        f.write('static const double rys_coef_host[RYS_NCOEF] = {\n')
        for a in range(0, len(coef), 4):
            f.write('  ' + ', '.join(v.hex() for v in coef[a:a + 4]) + ',\n')
        f.write('};\n')
        f.write('static const double rys_large_r_host[%d] = {\n  %s};\n'
                % (len(lr), ',\n  '.join(v.hex() for v in lr)))
        f.write('static const double rys_large_w_host[%d] = {\n  %s};\n'
                % (len(lw), ',\n  '.join(v.hex() for v in lw)))
    print('wrote', args.out, len(coef), 'coefficients')


if __name__ == '__main__':
    main()
