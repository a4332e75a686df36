"""Arbitrary-precision Rys roots and weights (mpmath), used offline to generate the GPU tables.

Rys quadrature for  int_0^1 f(t^2) exp(-x t^2) dt  with n nodes s_i = t_i^2 (the contract of
libcint's CINTrys_roots, src/rys_roots.c:57-122, and of its mpmath definition
scripts/rys_roots.py).  Method, written anew:
  * Boys moments F_m(x) = int_0^1 t^{2m} exp(-x t^2) dt from a convergent series for the top m
    and the stable downward recursion F_{m-1} = (2x F_m + e^{-x}) / (2m-1);
  * modified Chebyshev algorithm (Gautschi, "Orthogonal polynomials", 2004, sec. 2.1.7) with
    ordinary moments for the three-term recurrence of the orthogonal polynomials in s;
  * nodes by Newton iteration on p_n(s) started from the float64 Golub-Welsch nodes, weights
    by the Christoffel numbers 1 / sum_k p_k(s_i)^2 / h_k.
Large-x limit: positive Gauss-Hermite nodes y_i of H_{2n}: s_i = y_i^2/x, w_i = W_i/sqrt(x).
"""
import mpmath
import numpy as np

DPS = 60


def boys_moments(x, mmax):
    """F_0..F_mmax at x with mpmath precision (x is an mpf)."""
    ex = mpmath.exp(-x)
    # series: F_m(x) = e^{-x} sum_k (2x)^k / prod_{j=0..k} (2m+2j+1)
    m = mmax
    term = mpmath.mpf(1) / (2 * m + 1)
    s = term
    k = 0
    tiny = mpmath.mpf(10) ** (-(DPS + 5))
    while True:
        k += 1
        term = term * (2 * x) / (2 * m + 2 * k + 1)
        s += term
        if term < tiny * s:
            break
    F = [mpmath.mpf(0)] * (mmax + 1)
    F[mmax] = ex * s
    for mm in range(mmax, 0, -1):
        F[mm - 1] = (2 * x * F[mm] + ex) / (2 * mm - 1)
    return F


def recurrence(n, x):
    """alpha_k, beta_k (k < n) of the monic orthogonal polynomials for weight
    exp(-x s) s^{-1/2}/2 on s in [0,1] (i.e. exp(-x t^2) dt), from the moments F_k(x)."""
    mu = boys_moments(x, 2 * n)
    sig_prev = [mpmath.mpf(0)] * (2 * n + 1)
    sig = list(mu)
    alpha = [mu[1] / mu[0]]
    beta = [mu[0]]
    for k in range(1, n):
        new = [mpmath.mpf(0)] * (2 * n + 1)
        for l in range(k, 2 * n - k):
            new[l] = sig[l + 1] - alpha[k - 1] * sig[l] - beta[k - 1] * sig_prev[l]
        alpha.append(new[k + 1] / new[k] - sig[k] / sig[k - 1])
        beta.append(new[k] / sig[k - 1])
        sig_prev, sig = sig, new
    return alpha, beta


def _poly_all(alpha, beta, s, n):
    """p_0..p_n and p_n' at s (monic three-term recurrence)."""
    p = [mpmath.mpf(1), s - alpha[0]]
    dp = [mpmath.mpf(0), mpmath.mpf(1)]
    for k in range(1, n):
        p.append((s - alpha[k]) * p[k] - beta[k] * p[k - 1])
        dp.append(p[k] + (s - alpha[k]) * dp[k] - beta[k] * dp[k - 1])
    return p, dp


def rys_exact(n, x):
    """(s_i, w_i) as mpf lists, ascending s; s = t^2 in (0,1)."""
    with mpmath.workdps(DPS):
        x = mpmath.mpf(x)
        alpha, beta = recurrence(n, x)
        J = np.zeros((n, n))
        for k in range(n):
            J[k, k] = float(alpha[k])
            if k + 1 < n:
                J[k, k + 1] = J[k + 1, k] = float(mpmath.sqrt(beta[k + 1]))
        s0 = np.sort(np.linalg.eigvalsh(J))
        nodes = []
        for si in s0:
            s = mpmath.mpf(float(si))
            for _ in range(40):
                p, dp = _poly_all(alpha, beta, s, n)
                ds = p[n] / dp[n]
                s -= ds
                if abs(ds) < mpmath.mpf(10) ** (-(DPS - 8)) * abs(s):
                    break
            nodes.append(s)
        h = [beta[0]]
        for k in range(1, n):
            h.append(h[-1] * beta[k])
        weights = []
        for s in nodes:
            p, _ = _poly_all(alpha, beta, s, n)
            weights.append(1 / sum(p[k] ** 2 / h[k] for k in range(n)))
        return nodes, weights


def hermite_half(n):
    """Positive nodes y_i of H_{2n} (ascending) and their Gauss-Hermite weights, mpf."""
    with mpmath.workdps(DPS):
        m = 2 * n
        # Golub-Welsch start in float64, Newton refinement on the physicists' H_m
        J = np.zeros((m, m))
        for k in range(1, m):
            J[k - 1, k] = J[k, k - 1] = np.sqrt(k / 2.0)
        y0 = np.sort(np.linalg.eigvalsh(J))[n:]
        ys, ws = [], []
        for yf in y0:
            y = mpmath.mpf(float(yf))
            for _ in range(60):
                h0, h1 = mpmath.mpf(1), 2 * y
                for k in range(1, m):
                    h0, h1 = h1, 2 * y * h1 - 2 * k * h0
                # h1 = H_m, h0 = H_{m-1};  H_m' = 2m H_{m-1}
                dy = h1 / (2 * m * h0)
                y -= dy
                if abs(dy) < mpmath.mpf(10) ** (-(DPS - 8)):
                    break
            h0, h1 = mpmath.mpf(1), 2 * y
            for k in range(1, m):
                h0, h1 = h1, 2 * y * h1 - 2 * k * h0
            w = (2 ** (m - 1) * mpmath.factorial(m) * mpmath.sqrt(mpmath.pi)) / (m * m * h0 ** 2)
            ys.append(y)
            ws.append(w)
        return ys, ws
