"""The committed Rys tables (libcint_gb300/csrc/rys_tables.inc) evaluated on the host exactly as
the kernels do (Horner in y = 2(x - k) - 1, half-range Gauss-Hermite limit beyond x_max), against
60-digit values.  CPU only; needs mpmath (present where the tables are generated)."""
import os
import re
import sys

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(__file__)), 'libcint_gb300', 'csrc')


def _load():
    src = open(os.path.join(CSRC, 'rys_tables.inc')).read()

    def arr(name):
        m = re.search(name + r'\[[^\]]*\] = \{(.*?)\};', src, re.S)
        return [float.fromhex(t) if 'x' in t else float(t)
                for t in re.findall(r'[-+0-9a-fA-Fx.p]+', m.group(1))]
    deg = int(re.search(r'#define RYS_DEG (\d+)', src).group(1))
    h = float(re.search(r'#define RYS_H ([0-9.]+)', src).group(1))
    nmax = int(re.search(r'#define RYS_NMAX (\d+)', src).group(1))
    return (np.array(arr('rys_coef_host')), [int(v) for v in arr('rys_off_host')],
            [int(v) for v in arr('rys_nint_host')], np.array(arr('rys_large_r_host')),
            np.array(arr('rys_large_w_host')), deg, h, nmax)


def test_tables_against_60_digit_values():
    pytest.importorskip('mpmath')
    sys.path.insert(0, CSRC)
    import rys_exact as R
    coef, off, nint, lr, lw, deg, h, nmax = _load()
    rng = np.random.RandomState(5)
    for n in range(1, nmax + 1):
        xmax = h * nint[n]
        xs = list(rng.uniform(0, xmax, 12)) + list(rng.uniform(xmax, 400, 3)) + [0.0, xmax - 1e-9, xmax]
        for x in xs:
            if x >= xmax:
                o = n * (n - 1) // 2
                s, w = lr[o:o + n] / x, lw[o:o + n] / np.sqrt(x)
            else:
                k = int(x / h)
                y = 2 * (x - k * h) / h - 1
                s, w = np.zeros(n), np.zeros(n)
                for i in range(n):
                    b = off[n] + (k * n + i) * (deg + 1) * 2
                    cs, cw = coef[b:b + 2 * (deg + 1):2], coef[b + 1:b + 2 * (deg + 1):2]
                    a, c = cs[deg], cw[deg]
                    for j in range(deg - 1, -1, -1):
                        a, c = a * y + cs[j], c * y + cw[j]
                    s[i], w[i] = a, c
            se, we = R.rys_exact(n, x)
            f0 = float(sum(we))
            assert max(abs(float(p) - q) for p, q in zip(se, s)) < 1e-15, (n, x)
            assert max(abs(float(p) - q) for p, q in zip(we, w)) < 1e-15 * f0, (n, x)
