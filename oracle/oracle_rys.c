/*
 * CPU restatement of libcint 6.1.1's Rys-quadrature ERIs -- TEST INFRASTRUCTURE (the oracle).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load this library; the product
 * (libcintgpu.so) never does.  Every function cites the libcint code whose behaviour it
 * restates (paths relative to the libcint source tree).  The arithmetic is written anew:
 *   - Rys roots/weights by a discretised Stieltjes procedure + Golub-Welsch (independent of
 *     libcint's polynomial fits in src/rys_roots.c and of the GPU's Chebyshev tables);
 *   - VRR/HRR with the i and k centres as recurrence bases (libcint picks the larger l);
 *   - Cartesian -> real solid harmonics from the closed-form coefficients of Schlegel & Frisch
 *     (IJQC 54 (1995) 83), generated at run time rather than tabulated.
 * Screening, prefactors, component order, contraction layout and output layout follow libcint
 * exactly so the results agree element by element.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle_rys.h"

/* libcint include/cint.h.in:26-72 slot layout */
#define PTR_EXPCUTOFF   0
#define PTR_RANGE_OMEGA 8
#define PTR_COORD       1
#define ATM_SLOTS       6
#define ATOM_OF         0
#define ANG_OF          1
#define NPRIM_OF        2
#define NCTR_OF         3
#define PTR_EXP         5
#define PTR_COEFF       6
#define BAS_SLOTS       8

#define MAXROOTS 24
#define MAXL     8          /* per-shell ceiling supported by the oracle (l <= 7, +1 for ip1) */
#define MAXCART  36         /* (MAXL)(MAXL+1)/2 for l=7 */
#define NGL      200

static double gl_t[NGL], gl_w[NGL];   /* Gauss-Legendre on [0,1] */

/* Legendre nodes by Newton iteration on P_n (standard three-term recurrence). */
__attribute__((constructor)) static void init_gauss_legendre(void)
{
    const int n = NGL;
    for (int i = 0; i < (n + 1) / 2; i++) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5));
        double pp = 0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; j++) {
                double p3 = p2; p2 = p1;
                p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1);
            double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-16) break;
        }
        double w = 2.0 / ((1 - z * z) * pp * pp);
        /* map [-1,1] -> [0,1] */
        gl_t[i] = 0.5 * (1 - z);         gl_w[i] = 0.5 * w;
        gl_t[n - 1 - i] = 0.5 * (1 + z); gl_w[n - 1 - i] = 0.5 * w;
    }
}

/* Implicit QL on a symmetric tridiagonal matrix; d: diagonal (-> eigenvalues), e: e[i]
 * couples i,i+1 (e[n-1] ignored), z: n*n row-major eigenvectors (identity on input). */
static int tridiag_ql(int n, double *d, double *e, double *z)
{
    e[n - 1] = 0;
    for (int l = 0; l < n; l++) {
        int iter = 0, m;
        do {
            for (m = l; m < n - 1; m++) {
                double dd = fabs(d[m]) + fabs(d[m + 1]);
                if (fabs(e[m]) + dd == dd) break;
            }
            if (m != l) {
                if (iter++ == 100) return 1;
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = hypot(g, 1.0);
                g = d[m] - d[l] + e[l] / (g + (g >= 0 ? fabs(r) : -fabs(r)));
                double s = 1, c = 1, p = 0;
                int i;
                for (i = m - 1; i >= l; i--) {
                    double f = s * e[i], b = c * e[i];
                    r = hypot(f, g);
                    e[i + 1] = r;
                    if (r == 0.0) { d[i + 1] -= p; e[m] = 0; break; }
                    s = f / r; c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * b;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - b;
                    for (int k = 0; k < n; k++) {
                        f = z[k * n + i + 1];
                        z[k * n + i + 1] = s * z[k * n + i] + c * f;
                        z[k * n + i] = c * z[k * n + i] - s * f;
                    }
                }
                if (r == 0.0 && i >= l) continue;
                d[l] -= p; e[l] = g; e[m] = 0;
            }
        } while (m != l);
    }
    return 0;
}

/* Rys quadrature for weight exp(-x t^2) on t in [lower, 1] with nodes in s = t^2: lower = 0 is
 * the Coulomb operator (the contract of CINTrys_roots, src/rys_roots.c:57-122: u = s/(1-s),
 * sum w = F_0(x)); lower = sqrt(theta) the short-range erfc(omega r)/r one (the contract of
 * CINTsr_rys_roots, src/rys_roots.c:149-267, whose methods are not restated: the same discretised
 * Stieltjes procedure as for lower = 0 on the shorter interval). */
int oracle_rys_roots_range(int nroots, double x, double lower, double *u, double *w)
{
    if (nroots < 1 || nroots > MAXROOTS) return 1;
    /* integrand negligible beyond x (t^2 - lower^2) = K (K grows with the polynomial degree 4n) */
    double tmax = 1.0;
    double K = 80.0 + 8.0 * nroots;
    if (x * (1.0 - lower * lower) > K) tmax = sqrt(lower * lower + K / x);
    double s[NGL], W[NGL], q[NGL], qp[NGL], r[NGL];
    static const int M = NGL;
    double Q[MAXROOTS + 1][NGL];
    double mu0 = 0;
    const double span = tmax - lower;
    for (int j = 0; j < M; j++) {
        double t = lower + span * gl_t[j];
        s[j] = t * t;
        W[j] = span * gl_w[j] * exp(-x * t * t);
        mu0 += W[j];
    }
    double alpha[MAXROOTS], beta[MAXROOTS + 1];
    double inv = 1.0 / sqrt(mu0);
    for (int j = 0; j < M; j++) { q[j] = inv; qp[j] = 0; Q[0][j] = inv; }
    beta[0] = 0;
    for (int k = 0; k < nroots; k++) {
        double a = 0;
        for (int j = 0; j < M; j++) a += W[j] * s[j] * q[j] * q[j];
        alpha[k] = a;
        if (k == nroots - 1) break;
        double sb = sqrt(beta[k]);
        for (int j = 0; j < M; j++) r[j] = (s[j] - a) * q[j] - sb * qp[j];
        /* one pass of full re-orthogonalisation (Lanczos with reorthogonalisation) */
        for (int i = 0; i <= k; i++) {
            double dot = 0;
            for (int j = 0; j < M; j++) dot += W[j] * r[j] * Q[i][j];
            for (int j = 0; j < M; j++) r[j] -= dot * Q[i][j];
        }
        double nb = 0;
        for (int j = 0; j < M; j++) nb += W[j] * r[j] * r[j];
        beta[k + 1] = nb;
        double in = 1.0 / sqrt(nb);
        for (int j = 0; j < M; j++) { qp[j] = q[j]; q[j] = r[j] * in; Q[k + 1][j] = q[j]; }
    }
    double d[MAXROOTS], e[MAXROOTS], z[MAXROOTS * MAXROOTS];
    for (int i = 0; i < nroots; i++) {
        d[i] = alpha[i];
        e[i] = (i + 1 < nroots) ? sqrt(beta[i + 1]) : 0;
        for (int k = 0; k < nroots; k++) z[i * nroots + k] = (i == k);
    }
    if (tridiag_ql(nroots, d, e, z)) return 1;
    double wt[MAXROOTS];
    for (int i = 0; i < nroots; i++) wt[i] = mu0 * z[i] * z[i];  /* first eigenvector row */
    /* ascending nodes */
    for (int i = 1; i < nroots; i++) {
        double dv = d[i], wv = wt[i];
        int k = i - 1;
        while (k >= 0 && d[k] > dv) { d[k + 1] = d[k]; wt[k + 1] = wt[k]; k--; }
        d[k + 1] = dv; wt[k + 1] = wv;
    }
    for (int i = 0; i < nroots; i++) {
        u[i] = d[i] / (1.0 - d[i]);
        w[i] = wt[i];
    }
    return 0;
}

#ifdef ORACLE_TABLE_ROOTS
/* CPU timing build only (oracle_bench_fast, the CPU baseline legs of bench.py): the Coulomb roots
 * from the piecewise polynomial tables the GPU kernels use (rys_tables.inc: degree-10 pieces of
 * width 1 in x, Gauss-Hermite asymptotics beyond), instead of the Stieltjes procedure above,
 * which takes three quarters of the restatement's time.  The test oracle never defines this. */
#include "rys_tables.inc"
int oracle_rys_roots(int nroots, double x, double *u, double *w)
{
    if (nroots < 1 || nroots > RYS_NMAX) return oracle_rys_roots_range(nroots, x, 0.0, u, w);
    for (int r = 0; r < nroots; r++) {
        double s, wt;
        if (x >= RYS_H * rys_nint_host[nroots]) {
            const int o = nroots * (nroots - 1) / 2 + r;
            const double rs = 1.0 / sqrt(x);
            s = rys_large_r_host[o] * rs * rs;
            wt = rys_large_w_host[o] * rs;
        } else {
            const int k = (int)x;
            const double y = 2.0 * (x - k) - 1.0;
            const double *c = rys_coef_host + rys_off_host[nroots] + (size_t)((k * nroots + r) * (RYS_DEG + 1)) * 2;
            double a = c[2 * RYS_DEG], b = c[2 * RYS_DEG + 1];
            for (int j = RYS_DEG - 1; j >= 0; j--) {
                a = a * y + c[2 * j];
                b = b * y + c[2 * j + 1];
            }
            s = a;
            wt = b;
        }
        u[r] = s / (1.0 - s);
        w[r] = wt;
    }
    return 0;
}
#else
int oracle_rys_roots(int nroots, double x, double *u, double *w)
{
    return oracle_rys_roots_range(nroots, x, 0.0, u, w);
}
#endif

/* ------------------------------------------------------------------ cart -> sph */
static double fact(int n) { double f = 1; for (int i = 2; i <= n; i++) f *= i; return f; }
static double binom(int n, int k)
{
    if (k < 0 || k > n) return 0;
    return fact(n) / (fact(k) * fact(n - k));
}

/* Cartesian component order of CINTcart_comp (src/cint_bas.c:166-181): lx from l down to 0,
 * then ly from l-lx down to 0. */
static int cart_index(int l, int lx, int ly)
{
    int idx = 0;
    for (int x = l; x > lx; x--) idx += l - x + 1;
    return idx + (l - lx - ly);
}

/* Real solid harmonics r^l Y_lm, unit-sphere normalised, Condon-Shortley phase as libcint
 * (src/cart2sph.c:8-10 -> scripts/cart2sph.py).  Closed form of the Racah-normalised S_lm
 * times sqrt((2l+1)/4pi). Rows m = -l..l for l >= 2; identity for l = 0, 1. */
int oracle_cart2sph_coeff(int l, double *c)
{
    int nc = (l + 1) * (l + 2) / 2;
    if (l <= 1) {
        for (int i = 0; i < nc * nc; i++) c[i] = 0;
        for (int i = 0; i < nc; i++) c[i * nc + i] = 1;
        return nc;
    }
    int ns = 2 * l + 1;
    for (int i = 0; i < ns * nc; i++) c[i] = 0;
    double unit = sqrt((2 * l + 1) / (4 * M_PI));
    for (int m = -l; m <= l; m++) {
        int am = abs(m);
        double N = sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0))
                   / (pow(2.0, am) * fact(l));
        int row = m + l;
        for (int t = 0; t <= (l - am) / 2; t++) {
            for (int uu = 0; uu <= t; uu++) {
                /* 2v runs over even values (m >= 0) or odd values (m < 0) up to |m| */
                for (int v2 = (m < 0 ? 1 : 0); v2 <= am; v2 += 2) {
                    int vm2 = (m < 0 ? 1 : 0);
                    int sgn_exp = t + (v2 - vm2) / 2;
                    double C = ((sgn_exp & 1) ? -1.0 : 1.0) * pow(0.25, t) * binom(l, t)
                             * binom(l - t, am + t) * binom(t, uu) * binom(am, v2);
                    int px = 2 * t + am - 2 * uu - v2;
                    int py = 2 * uu + v2;
                    int pz = l - 2 * t - am;
                    if (px < 0 || py < 0 || pz < 0) continue;
                    c[row * nc + cart_index(l, px, py)] += unit * N * C;
                }
            }
        }
    }
    return ns;
}

/* ------------------------------------------------------------------ integral engine */
typedef struct {
    int l[4];          /* angular momentum per slot (slot 3 is a dummy s shell for 3c2e, slots 1
                          and 3 for 2c2e) */
    int lc[4];         /* g-array ceilings, l + derivative increment */
    int nprim[4], nctr[4];
    double r[4][3];
    const double *ex[4], *cf[4];
    double dummy_exp, dummy_cf;
    double common;
    double expcutoff;
    double omega;      /* env[PTR_RANGE_OMEGA]: > 0 long-range erf(omega r)/r Coulomb */
    int three_center;  /* 0 int2e, 1 int3c2e, 2 int2c2e */
    int deriv_i;       /* 1 for a nabla on one shell (ip1: i, ip2: k) */
    int dslot;         /* the nabla's shell slot: 0 (i) or 2 (k) */
    int nroots;
} OEnv;

static double common_fac_sp(int l)   /* src/g1e.c:565-572 */
{
    if (l == 0) return 0.282094791773878143;
    if (l == 1) return 0.488602511902919921;
    return 1.0;
}

static void load_shell(OEnv *E, int slot, int sh, int *atm, int *bas, double *env)
{
    int *b = bas + BAS_SLOTS * sh;
    E->l[slot] = b[ANG_OF];
    E->nprim[slot] = b[NPRIM_OF];
    E->nctr[slot] = b[NCTR_OF];
    const double *r = env + atm[ATM_SLOTS * b[ATOM_OF] + PTR_COORD];
    E->r[slot][0] = r[0]; E->r[slot][1] = r[1]; E->r[slot][2] = r[2];
    E->ex[slot] = env + b[PTR_EXP];
    E->cf[slot] = env + b[PTR_COEFF];
}

/* CINTinit_int2e_EnvVars (src/g2e.c:21-172) / CINTinit_int3c2e_EnvVars (src/g3c2e.c:21-132) /
 * CINTinit_int2c2e_EnvVars (src/g2c2e.c:16-56): int2c2e's (i|k) is (i s0|k s0) with two dummy
 * zero-exponent unit s shells, the common factor of i and k only and no +1 on the cutoff */
static void init_env(OEnv *E, int *shls, int *atm, int *bas, double *env, int three, int dinc,
                     int dslot)
{
    memset(E, 0, sizeof(*E));
    E->three_center = three;
    E->omega = env[PTR_RANGE_OMEGA];
    if (three == 2) {
        load_shell(E, 0, shls[0], atm, bas, env);
        load_shell(E, 2, shls[1], atm, bas, env);
        E->dummy_exp = 0; E->dummy_cf = 1;
        const int units[2] = {1, 3};
        for (int u = 0; u < 2; u++) {
            const int s = units[u];
            E->l[s] = 0; E->nprim[s] = 1; E->nctr[s] = 1;
            memcpy(E->r[s], E->r[s - 1], sizeof(double) * 3);
            E->ex[s] = &E->dummy_exp; E->cf[s] = &E->dummy_cf;
        }
        E->common = M_PI * M_PI * M_PI * 2 / 1.7724538509055160272981674833411451
                  * common_fac_sp(E->l[0]) * common_fac_sp(E->l[2]);
        E->expcutoff = env[PTR_EXPCUTOFF] == 0 ? 60 : fmax(40, env[PTR_EXPCUTOFF]);
        E->deriv_i = dinc;
        for (int s = 0; s < 4; s++) E->lc[s] = E->l[s];
        E->lc[0] += dinc;
        E->nroots = (E->lc[0] + E->lc[2]) / 2 + 1;
        return;
    }
    load_shell(E, 0, shls[0], atm, bas, env);
    load_shell(E, 1, shls[1], atm, bas, env);
    load_shell(E, 2, shls[2], atm, bas, env);
    if (three) {
        E->l[3] = 0; E->nprim[3] = 1; E->nctr[3] = 1;
        memcpy(E->r[3], E->r[2], sizeof(double) * 3);
        E->dummy_exp = 0; E->dummy_cf = 1;
        E->ex[3] = &E->dummy_exp; E->cf[3] = &E->dummy_cf;
        E->common = M_PI * M_PI * M_PI * 2 / 1.7724538509055160272981674833411451
                  * common_fac_sp(E->l[0]) * common_fac_sp(E->l[1]) * common_fac_sp(E->l[2]);
        E->expcutoff = env[PTR_EXPCUTOFF] == 0 ? 60 : fmax(40, env[PTR_EXPCUTOFF]);
    } else {
        load_shell(E, 3, shls[3], atm, bas, env);
        E->common = M_PI * M_PI * M_PI * 2 / 1.7724538509055160272981674833411451
                  * common_fac_sp(E->l[0]) * common_fac_sp(E->l[1])
                  * common_fac_sp(E->l[2]) * common_fac_sp(E->l[3]);
        E->expcutoff = env[PTR_EXPCUTOFF] == 0 ? 60 : fmax(40, env[PTR_EXPCUTOFF]) + 1;
    }
    E->deriv_i = dinc;
    E->dslot = dslot;
    for (int s = 0; s < 4; s++) E->lc[s] = E->l[s];
    E->lc[dslot] += dinc;   /* libcint's ng IINC / KINC (src/autocode/grad2.c, int3c2e.c) */
    E->nroots = (E->lc[0] + E->lc[1] + E->lc[2] + E->lc[3]) / 2 + 1;
}

static int ncart(int l) { return (l + 1) * (l + 2) / 2; }

/* g arrays: G[coord][root][i][j][k][l] flattened with extents lc+1 */
typedef struct {
    int di, dj, dk, dl;   /* extents */
    int n;                /* nroots */
    double *g;            /* 3 * n * di*dj*dk*dl */
} GArr;

#define GIDX(G, c, r, i, j, k, l) \
    ((((((size_t)(c) * (G)->n + (r)) * (G)->di + (i)) * (G)->dj + (j)) * (G)->dk + (k)) * (G)->dl + (l))

/* CINTg0_2e (src/g2e.c:4425-4545) + CINTg0_2e_2d (VRR, :272-421) + HRR (:428-693), written
 * with i and k as the recurrence bases.  P, Q: pair centres; aij, akl: pair exponents; cutoff:
 * the primitive quartet's remaining screening budget (expcutoff - cce_ij - cce_kl).  Returns 1
 * when the short-range operator screens the primitive quartet out, -1 on failure. */
static int g0_2e(const OEnv *E, GArr *G, const double *P, const double *Q,
                 double aij, double akl, double fac, double cutoff)
{
    const int n = E->nroots;
    double u[MAXROOTS], w[MAXROOTS];
    double PQ[3] = {P[0] - Q[0], P[1] - Q[1], P[2] - Q[2]};
    double rr = PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2];
    double a1 = aij * akl;
    double a0 = a1 / (aij + akl);
    double fac1 = sqrt(a0 / (a1 * a1 * a1)) * fac;
    double x = a0 * rr;
    double theta = 1, lower = 0;
    if (E->omega < 0) {
        /* short-range erfc(omega r)/r (src/g2e.c:4447-4476): the Rys weight restricted to
         * t >= sqrt(theta), theta = omega^2/(omega^2 + a0); a primitive quartet whose theta x
         * exceeds its screening budget (or 40) is dropped, as libcint does */
        theta = E->omega * E->omega / (E->omega * E->omega + a0);
        if (theta * x > cutoff || theta * x > 40.0) return 1;
        lower = sqrt(theta);
    } else if (E->omega > 0) {
        /* long-range Coulomb erf(omega r)/r (src/g2e.c:4477-4492): the Rys quadrature of
         * x' = theta x with theta = omega^2/(omega^2 + a0), weights times sqrt(theta), and every
         * node mapped to t^2 -> theta t^2, i.e. u -> theta u / (1 + u - theta u) */
        theta = E->omega * E->omega / (E->omega * E->omega + a0);
        x *= theta;
        fac1 *= sqrt(theta);
    }
    if (lower > 0 ? oracle_rys_roots_range(n, x, lower, u, w) : oracle_rys_roots(n, x, u, w)) return -1;
    if (E->omega > 0)
        for (int r = 0; r < n; r++) u[r] = theta * u[r] / (1 + u[r] - theta * u[r]);
    const int nmax = E->lc[0] + E->lc[1];
    const int mmax = E->lc[2] + E->lc[3];
    /* 2D table per root and coordinate: T[n][m] */
    double T[2 * MAXL + 1][2 * MAXL + 1];
    double PA[3], QC[3], AB[3], CD[3];
    for (int c = 0; c < 3; c++) {
        PA[c] = P[c] - E->r[0][c];
        QC[c] = Q[c] - E->r[2][c];
        AB[c] = E->r[0][c] - E->r[1][c];
        CD[c] = E->r[2][c] - E->r[3][c];
    }
    for (int r = 0; r < n; r++) {
        double u2 = a0 * u[r];
        double tmp4 = .5 / (u2 * (aij + akl) + a1);
        double b00 = u2 * tmp4;
        double b10 = b00 + tmp4 * akl;
        double b01 = b00 + tmp4 * aij;
        double tmp2 = 2. * b00 * akl;
        double tmp3 = 2. * b00 * aij;
        for (int c = 0; c < 3; c++) {
            double c00 = PA[c] - tmp2 * PQ[c];
            double c0p = QC[c] + tmp3 * PQ[c];
            T[0][0] = (c == 2) ? w[r] * fac1 : 1.0;
            for (int a = 0; a < nmax; a++)
                T[a + 1][0] = c00 * T[a][0] + (a ? a * b10 * T[a - 1][0] : 0);
            for (int m = 0; m < mmax; m++) {
                for (int a = 0; a <= nmax; a++) {
                    double v = c0p * T[a][m];
                    if (m) v += m * b01 * T[a][m - 1];
                    if (a) v += a * b00 * T[a - 1][m];
                    T[a][m + 1] = v;
                }
            }
            /* HRR: (a, b+1| = (a+1, b| + AB (a, b|, same for |c, d) */
            double H[2 * MAXL + 1][MAXL + 1][2 * MAXL + 1][MAXL + 1];
            for (int a = 0; a <= nmax; a++)
                for (int m = 0; m <= mmax; m++) H[a][0][m][0] = T[a][m];
            for (int b = 1; b <= E->lc[1]; b++)
                for (int a = 0; a <= nmax - b; a++)
                    for (int m = 0; m <= mmax; m++)
                        H[a][b][m][0] = H[a + 1][b - 1][m][0] + AB[c] * H[a][b - 1][m][0];
            for (int d = 1; d <= E->lc[3]; d++)
                for (int m = 0; m <= mmax - d; m++)
                    for (int a = 0; a <= E->lc[0]; a++)
                        for (int b = 0; b <= E->lc[1]; b++)
                            H[a][b][m][d] = H[a][b][m + 1][d - 1] + CD[c] * H[a][b][m][d - 1];
            for (int a = 0; a <= E->lc[0]; a++)
                for (int b = 0; b <= E->lc[1]; b++)
                    for (int k = 0; k <= E->lc[2]; k++)
                        for (int d = 0; d <= E->lc[3]; d++)
                            G->g[GIDX(G, c, r, a, b, k, d)] = H[a][b][k][d];
        }
    }
    return 0;
}

static void cart_comp(int l, int *nx, int *ny, int *nz)   /* CINTcart_comp order */
{
    int inc = 0;
    for (int lx = l; lx >= 0; lx--)
        for (int ly = l - lx; ly >= 0; ly--) {
            nx[inc] = lx; ny[inc] = ly; nz[inc] = l - lx - ly; inc++;
        }
}

/* Primitive-quartet contribution: CINTgout2e (src/cint2e.c:961-1183) for ncomp = 1, or
 * CINTgout2e_int2e_ip1 + CINTnabla1i_2e (src/autocode/grad2.c:19-68, src/g2e.c:4550-4591) for
 * ncomp = 3.  Component order n = i + nfi*(k + nfk*(l + nfl*j)) as CINTg2e_index_xyz. */
static void gout(const OEnv *E, const GArr *G, double ai, double *out, int ncomp)
{
    int nx[4][MAXCART], ny[4][MAXCART], nz[4][MAXCART];
    int nf[4];
    for (int s = 0; s < 4; s++) { cart_comp(E->l[s], nx[s], ny[s], nz[s]); nf[s] = ncart(E->l[s]); }
    const int n = E->nroots;
    /* offsets of root 0 per axis; consecutive roots are rs apart (GIDX layout) */
    const size_t rs = (size_t)G->di * G->dj * G->dk * G->dl;
    size_t idx = 0;
    for (int j = 0; j < nf[1]; j++)
    for (int l = 0; l < nf[3]; l++)
    for (int k = 0; k < nf[2]; k++)
    for (int i = 0; i < nf[0]; i++, idx++) {
        int ix = nx[0][i], iy = ny[0][i], iz = nz[0][i];
        const double *px = G->g + GIDX(G, 0, 0, ix, nx[1][j], nx[2][k], nx[3][l]);
        const double *py = G->g + GIDX(G, 1, 0, iy, ny[1][j], ny[2][k], ny[3][l]);
        const double *pz = G->g + GIDX(G, 2, 0, iz, nz[1][j], nz[2][k], nz[3][l]);
        double s0 = 0, sx = 0, sy = 0, sz = 0, h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int r = 0; r < n; r++) {
            double gx = px[r * rs];
            double gy = py[r * rs];
            double gz = pz[r * rs];
            if (ncomp == 1) {
                s0 += gx * gy * gz;
            } else if (ncomp == 9) {
                /* two nablas on i (libcint int2e_ipip1, src/autocode/hess.c:1124-1170):
                 * D g(i) = i g(i-1) - 2a g(i+1), D D g(i) = i(i-1) g(i-2) - 2a(2i+1) g(i)
                 * + 4a^2 g(i+2); component 3p + q = D_p D_q (one D per axis, D D on one) */
                const int ii[3] = {ix, iy, iz};
                const int jj[3] = {nx[1][j], ny[1][j], nz[1][j]};
                const int kk[3] = {nx[2][k], ny[2][k], nz[2][k]};
                const int ll[3] = {nx[3][l], ny[3][l], nz[3][l]};
                double g0[3], g1[3], g2[3];
                for (int c = 0; c < 3; c++) {
                    const int a = ii[c];
                    double v = G->g[GIDX(G, c, r, a, jj[c], kk[c], ll[c])];
                    double vp = G->g[GIDX(G, c, r, a + 1, jj[c], kk[c], ll[c])];
                    double vpp = G->g[GIDX(G, c, r, a + 2, jj[c], kk[c], ll[c])];
                    double vm = a >= 1 ? G->g[GIDX(G, c, r, a - 1, jj[c], kk[c], ll[c])] : 0;
                    double vmm = a >= 2 ? G->g[GIDX(G, c, r, a - 2, jj[c], kk[c], ll[c])] : 0;
                    g0[c] = v;
                    g1[c] = a * vm - 2 * ai * vp;
                    g2[c] = a * (a - 1) * vmm - 2 * ai * (2 * a + 1) * v + 4 * ai * ai * vpp;
                }
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++) {
                        double t = 1;
                        for (int c = 0; c < 3; c++)
                            t *= (c == p && c == q) ? g2[c] : ((c == p || c == q) ? g1[c] : g0[c]);
                        h[3 * p + q] += t;
                    }
            } else if (E->dslot == 0) {
                /* f(i) = i g(i-1) - 2 a_i g(i+1)   (CINTnabla1i_2e, src/g2e.c:4550-4591) */
                double fx = -2 * ai * G->g[GIDX(G, 0, r, ix + 1, nx[1][j], nx[2][k], nx[3][l])];
                double fy = -2 * ai * G->g[GIDX(G, 1, r, iy + 1, ny[1][j], ny[2][k], ny[3][l])];
                double fz = -2 * ai * G->g[GIDX(G, 2, r, iz + 1, nz[1][j], nz[2][k], nz[3][l])];
                if (ix) fx += ix * G->g[GIDX(G, 0, r, ix - 1, nx[1][j], nx[2][k], nx[3][l])];
                if (iy) fy += iy * G->g[GIDX(G, 1, r, iy - 1, ny[1][j], ny[2][k], ny[3][l])];
                if (iz) fz += iz * G->g[GIDX(G, 2, r, iz - 1, nz[1][j], nz[2][k], nz[3][l])];
                sx += fx * gy * gz;
                sy += gx * fy * gz;
                sz += gx * gy * fz;
            } else {
                /* f(k) = k g(k-1) - 2 a_k g(k+1)   (CINTnabla1k_2e, src/g2e.c:4651-4701) */
                const int kx = nx[2][k], ky = ny[2][k], kz = nz[2][k];
                double fx = -2 * ai * G->g[GIDX(G, 0, r, ix, nx[1][j], kx + 1, nx[3][l])];
                double fy = -2 * ai * G->g[GIDX(G, 1, r, iy, ny[1][j], ky + 1, ny[3][l])];
                double fz = -2 * ai * G->g[GIDX(G, 2, r, iz, nz[1][j], kz + 1, nz[3][l])];
                if (kx) fx += kx * G->g[GIDX(G, 0, r, ix, nx[1][j], kx - 1, nx[3][l])];
                if (ky) fy += ky * G->g[GIDX(G, 1, r, iy, ny[1][j], ky - 1, ny[3][l])];
                if (kz) fz += kz * G->g[GIDX(G, 2, r, iz, nz[1][j], kz - 1, nz[3][l])];
                sx += fx * gy * gz;
                sy += gx * fy * gz;
                sz += gx * gy * fz;
            }
        }
        if (ncomp == 1) out[idx] = s0;
        else if (ncomp == 9) for (int c = 0; c < 9; c++) out[idx * 9 + c] = h[c];
        else { out[idx * 3 + 0] = sx; out[idx * 3 + 1] = sy; out[idx * 3 + 2] = sz; }
    }
}

/* Primitive screening data of CINTset_pairdata (src/optimizer.c:288-342). */
typedef struct { double r[3]; double e; double cce; } OPair;

static void log_maxc(const double *c, int nprim, int nctr, double *out)   /* :248-259 */
{
    for (int ip = 0; ip < nprim; ip++) {
        double m = 0;
        for (int i = 0; i < nctr; i++) m = fmax(m, fabs(c[i * nprim + ip]));
        out[ip] = log(m);
    }
}

static int set_pairdata(OPair *pd, const double *ai, const double *aj, const double *ri,
                        const double *rj, const double *lci, const double *lcj, int li_c, int lj_c,
                        int ip_n, int jp_n, double expcutoff)
{
    double rr = (ri[0] - rj[0]) * (ri[0] - rj[0]) + (ri[1] - rj[1]) * (ri[1] - rj[1])
              + (ri[2] - rj[2]) * (ri[2] - rj[2]);
    double aij = ai[ip_n - 1] + aj[jp_n - 1];
    double log_rr = 1.7 - 1.5 * log(aij);
    int lij = li_c + lj_c;
    if (lij > 0) log_rr += lij * log(sqrt(rr) + 1.);
    int empty = 1;
    for (int n = 0, jp = 0; jp < jp_n; jp++)
        for (int ip = 0; ip < ip_n; ip++, n++) {
            double inv = 1 / (ai[ip] + aj[jp]);
            double eij = rr * ai[ip] * aj[jp] * inv;
            double cce = eij - log_rr - lci[ip] - lcj[jp];
            pd[n].cce = cce;
            if (cce < expcutoff) {
                empty = 0;
                double wj = aj[jp] * inv;
                for (int c = 0; c < 3; c++) pd[n].r[c] = ri[c] + wj * (rj[c] - ri[c]);
                pd[n].e = exp(-eij);
            } else {
                pd[n].r[0] = pd[n].r[1] = pd[n].r[2] = 1e18;
                pd[n].e = 0;
            }
        }
    return empty;
}

/* Contracted quartet in Cartesian components, layout of CINT2e_loop_nopt
 * (src/cint2e.c:57-269) and CINT3c2e_loop_nopt (src/cint3c2e.c:56-212):
 * gctr[comp][lc][kc][jc][ic][nf]. Returns 1 if any primitive quartet survived. */
static int contracted(const OEnv *E, double *gctr, int ncomp)
{
    const int nf = ncart(E->l[0]) * ncart(E->l[1]) * ncart(E->l[2]) * ncart(E->l[3]);
    const int nc = E->nctr[0] * E->nctr[1] * E->nctr[2] * E->nctr[3];
    memset(gctr, 0, sizeof(double) * (size_t)nf * nc * ncomp);
    double lci[64], lcj[64], lck[64], lcl[64];
    log_maxc(E->cf[0], E->nprim[0], E->nctr[0], lci);
    log_maxc(E->cf[1], E->nprim[1], E->nctr[1], lcj);
    log_maxc(E->cf[2], E->nprim[2], E->nctr[2], lck);
    log_maxc(E->cf[3], E->nprim[3], E->nctr[3], lcl);
    OPair *pij = malloc(sizeof(OPair) * E->nprim[0] * E->nprim[1]);
    if (E->three_center == 2) {
        /* CINT2c2e_loop_nopt (src/cint2c2e.c:58-150): no primitive screening */
        for (int ip = 0; ip < E->nprim[0]; ip++) {
            memcpy(pij[ip].r, E->r[0], sizeof(double) * 3);
            pij[ip].e = 1.0;
            pij[ip].cce = -HUGE_VAL;
        }
    } else if (set_pairdata(pij, E->ex[0], E->ex[1], E->r[0], E->r[1], lci, lcj, E->lc[0], E->lc[1],
                            E->nprim[0], E->nprim[1], E->expcutoff)) {
        free(pij);
        return 0;
    }
    GArr G;
    G.di = E->lc[0] + 1; G.dj = E->lc[1] + 1; G.dk = E->lc[2] + 1; G.dl = E->lc[3] + 1;
    G.n = E->nroots;
    G.g = malloc(sizeof(double) * 3 * G.n * G.di * G.dj * G.dk * G.dl);
    double *gp = malloc(sizeof(double) * nf * ncomp);
    const double *rk = E->r[2], *rl = E->r[3];
    double rr_kl = (rk[0] - rl[0]) * (rk[0] - rl[0]) + (rk[1] - rl[1]) * (rk[1] - rl[1])
                 + (rk[2] - rl[2]) * (rk[2] - rl[2]);
    double log_rr_kl = 1.7 - 1.5 * log(E->ex[2][E->nprim[2] - 1] + E->ex[3][E->nprim[3] - 1]);
    int lkl = E->lc[2] + E->lc[3];
    if (lkl > 0) log_rr_kl += lkl * log(sqrt(rr_kl) + 1.);
    int empty = 1;
    for (int lp = 0; lp < E->nprim[3]; lp++)
    for (int kp = 0; kp < E->nprim[2]; kp++) {
        double ak = E->ex[2][kp], al = E->ex[3][lp];
        double akl = ak + al;
        double Q[3], ekl, eijcutoff;
        if (E->three_center) {
            memcpy(Q, rk, sizeof(Q));
            ekl = 1.0;
            eijcutoff = E->expcutoff;
        } else {
            double e = rr_kl * ak * al / akl;
            double cce = e - log_rr_kl - lck[kp] - lcl[lp];
            if (cce > E->expcutoff) continue;
            for (int c = 0; c < 3; c++) Q[c] = (ak * rk[c] + al * rl[c]) / akl;
            eijcutoff = E->expcutoff - cce;
            ekl = exp(-e);
        }
        for (int jp = 0; jp < E->nprim[1]; jp++)
        for (int ip = 0; ip < E->nprim[0]; ip++) {
            const OPair *pd = pij + jp * E->nprim[0] + ip;
            if (pd->cce > eijcutoff) continue;
            double aij = E->ex[0][ip] + E->ex[1][jp];
            double fac = E->common * pd->e * ekl;
            const int rc = g0_2e(E, &G, pd->r, Q, aij, akl, fac, eijcutoff - pd->cce);
            if (rc < 0) { empty = 1; goto done; }
            if (rc > 0) continue;
            gout(E, &G, E->dslot == 2 ? ak : E->ex[0][ip], gp, ncomp);
            empty = 0;
            /* prim -> contracted for every contraction pattern (src/g1e.c:530-559) */
            for (int lc_ = 0; lc_ < E->nctr[3]; lc_++)
            for (int kc = 0; kc < E->nctr[2]; kc++)
            for (int jc = 0; jc < E->nctr[1]; jc++)
            for (int ic = 0; ic < E->nctr[0]; ic++) {
                double cc = E->cf[0][ic * E->nprim[0] + ip] * E->cf[1][jc * E->nprim[1] + jp]
                          * E->cf[2][kc * E->nprim[2] + kp] * E->cf[3][lc_ * E->nprim[3] + lp];
                size_t base = (size_t)nf * (ic + E->nctr[0] * (jc + E->nctr[1] * (kc + E->nctr[2] * lc_)));
                for (int comp = 0; comp < ncomp; comp++) {
                    double *dst = gctr + (size_t)comp * nf * nc + base;
                    for (int t = 0; t < nf; t++) dst[t] += cc * gp[t * ncomp + comp];
                }
            }
        }
    }
done:
    free(gp); free(G.g); free(pij);
    return !empty;
}

/* c2s_sph_2e1 / c2s_cart_2e1 (src/cart2sph.c:5324-5383, 5845-5872) + dcopy_iklj (:4558-4674)
 * + c2s_dset0 (:4707-4735): transform each contracted block and write
 * out[i + ni*(j + nj*(k + nk*l))] with leading dimensions dims. */
static void write_out(const OEnv *E, const double *gctr, double *out, int *dims, int sph,
                      int ncomp, int nonempty)
{
    int nfs[4], nds[4];
    double *C[4];
    for (int s = 0; s < 4; s++) {
        nfs[s] = ncart(E->l[s]);
        nds[s] = sph ? (E->l[s] <= 1 ? nfs[s] : 2 * E->l[s] + 1) : nfs[s];
        C[s] = malloc(sizeof(double) * nds[s] * nfs[s]);
        if (sph) oracle_cart2sph_coeff(E->l[s], C[s]);
        else { for (int a = 0; a < nds[s] * nfs[s]; a++) C[s][a] = 0;
               for (int a = 0; a < nfs[s]; a++) C[s][a * nfs[s] + a] = 1; }
    }
    int counts[4];
    for (int s = 0; s < 4; s++) counts[s] = nds[s] * E->nctr[s];
    int d[4];
    if (dims && E->three_center == 2) { d[0] = dims[0]; d[1] = 1; d[2] = dims[1]; d[3] = 1; }
    else if (dims) { d[0] = dims[0]; d[1] = dims[1]; d[2] = dims[2]; d[3] = E->three_center ? 1 : dims[3]; }
    else memcpy(d, counts, sizeof(d));
    size_t nout = (size_t)d[0] * d[1] * d[2] * d[3];
    const int nf = nfs[0] * nfs[1] * nfs[2] * nfs[3];
    const int nc = E->nctr[0] * E->nctr[1] * E->nctr[2] * E->nctr[3];
    for (int comp = 0; comp < ncomp; comp++) {
        double *o = out + comp * nout;
        for (int lc_ = 0; lc_ < E->nctr[3]; lc_++)
        for (int kc = 0; kc < E->nctr[2]; kc++)
        for (int jc = 0; jc < E->nctr[1]; jc++)
        for (int ic = 0; ic < E->nctr[0]; ic++) {
            const double *g = gctr + (size_t)comp * nf * nc
                + (size_t)nf * (ic + E->nctr[0] * (jc + E->nctr[1] * (kc + E->nctr[2] * lc_)));
            for (int ls = 0; ls < nds[3]; ls++)
            for (int ks = 0; ks < nds[2]; ks++)
            for (int js = 0; js < nds[1]; js++)
            for (int is = 0; is < nds[0]; is++) {
                double v = 0;
                if (nonempty) {
                    for (int j = 0; j < nfs[1]; j++) {
                        double cj = C[1][js * nfs[1] + j];
                        if (cj == 0) continue;
                        for (int l = 0; l < nfs[3]; l++) {
                            double cl = C[3][ls * nfs[3] + l];
                            if (cl == 0) continue;
                            for (int k = 0; k < nfs[2]; k++) {
                                double ck = C[2][ks * nfs[2] + k];
                                if (ck == 0) continue;
                                for (int i = 0; i < nfs[0]; i++) {
                                    double ci = C[0][is * nfs[0] + i];
                                    if (ci == 0) continue;
                                    v += ci * ck * cl * cj * g[i + nfs[0] * (k + nfs[2] * (l + nfs[3] * j))];
                                }
                            }
                        }
                    }
                }
                size_t oi = (size_t)(ic * nds[0] + is)
                          + (size_t)d[0] * ((jc * nds[1] + js)
                          + (size_t)d[1] * ((kc * nds[2] + ks) + (size_t)d[2] * (lc_ * nds[3] + ls)));
                o[oi] = v;
            }
        }
    }
    for (int s = 0; s < 4; s++) free(C[s]);
}

static int driver(double *out, int *dims, int *shls, int *atm, int *bas, double *env,
                  int three, int dinc, int sph, int dslot)
{
    OEnv E;
    init_env(&E, shls, atm, bas, env, three, dinc, dslot);

    int ncomp = dinc == 2 ? 9 : (dinc ? 3 : 1);
    int nf = ncart(E.l[0]) * ncart(E.l[1]) * ncart(E.l[2]) * ncart(E.l[3]);
    int nc = E.nctr[0] * E.nctr[1] * E.nctr[2] * E.nctr[3];
    if (out == NULL) {
        /* a cache size query: the oracle needs no cache, report a harmless positive size */
        return nf * nc * ncomp + 1;
    }
    double *gctr = malloc(sizeof(double) * (size_t)nf * nc * ncomp);
    int nonempty = contracted(&E, gctr, ncomp);
    write_out(&E, gctr, out, dims, sph, ncomp, nonempty);
    free(gctr);
    return nonempty;
}

int oracle_int2e_sph(double *out, int *dims, int *shls, int *atm, int natm,
                     int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 0, 1, 0); }
int oracle_int2e_cart(double *out, int *dims, int *shls, int *atm, int natm,
                      int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 0, 0, 0); }
int oracle_int2e_ip1_sph(double *out, int *dims, int *shls, int *atm, int natm,
                         int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 1, 1, 0); }
int oracle_int2e_ip1_cart(double *out, int *dims, int *shls, int *atm, int natm,
                          int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 1, 0, 0); }
int oracle_int3c2e_sph(double *out, int *dims, int *shls, int *atm, int natm,
                       int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 1, 0, 1, 0); }
int oracle_int3c2e_cart(double *out, int *dims, int *shls, int *atm, int natm,
                        int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 1, 0, 0, 0); }
int oracle_int2c2e_sph(double *out, int *dims, int *shls, int *atm, int natm,
                       int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 2, 0, 1, 0); }
int oracle_int2c2e_cart(double *out, int *dims, int *shls, int *atm, int natm,
                        int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 2, 0, 0, 0); }

int oracle_int2e_ip2_sph(double *out, int *dims, int *shls, int *atm, int natm,
                         int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 1, 1, 2); }
int oracle_int2e_ip2_cart(double *out, int *dims, int *shls, int *atm, int natm,
                          int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 1, 0, 2); }
int oracle_int3c2e_ip1_sph(double *out, int *dims, int *shls, int *atm, int natm,
                           int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 1, 1, 1, 0); }
int oracle_int3c2e_ip1_cart(double *out, int *dims, int *shls, int *atm, int natm,
                            int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 1, 1, 0, 0); }
int oracle_int3c2e_ip2_sph(double *out, int *dims, int *shls, int *atm, int natm,
                           int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 1, 1, 1, 2); }
int oracle_int3c2e_ip2_cart(double *out, int *dims, int *shls, int *atm, int natm,
                            int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 1, 1, 0, 2); }

int oracle_int2e_ipip1_sph(double *out, int *dims, int *shls, int *atm, int natm,
                           int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 2, 1, 0); }
int oracle_int2e_ipip1_cart(double *out, int *dims, int *shls, int *atm, int natm,
                            int *bas, int nbas, double *env, void *opt, double *cache)
{ (void)natm; (void)nbas; (void)opt; (void)cache; return driver(out, dims, shls, atm, bas, env, 0, 2, 0, 0); }

double oracle_int2e_sph_list(const int *quartets, long nq, double *out, const long *offsets,
                             int *atm, int natm, int *bas, int nbas, double *env, int nthreads)
{
    double t0 = 0, t1 = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    t0 = omp_get_wtime();
#endif
    long max_block = 0;
    for (long q = 0; q < nq; q++) {
        const int *s = quartets + 4 * q;
        long n = 1;
        for (int a = 0; a < 4; a++) {
            int *b = bas + BAS_SLOTS * s[a];
            n *= (long)(b[ANG_OF] * 2 + 1) * b[NCTR_OF];
        }
        if (n > max_block) max_block = n;
    }
#pragma omp parallel
    {
        double *scratch = malloc(sizeof(double) * (max_block > 0 ? max_block : 1));
#pragma omp for schedule(dynamic, 2)
        for (long q = 0; q < nq; q++) {
            double *dst = out ? out + offsets[q] : scratch;
            oracle_int2e_sph(dst, NULL, (int *)(quartets + 4 * q), atm, natm, bas, nbas, env,
                             NULL, NULL);
        }
        free(scratch);
    }
#ifdef _OPENMP
    t1 = omp_get_wtime();
#endif
    return t1 - t0;
}

/* Evaluate n items of one kind (which: 0 int2e_sph, 1 int2e_cart, 2 int2e_ip1_sph, 3 int2e_ip1_cart,
 * 4 int3c2e_sph, 5 int3c2e_cart, 6 int2c2e_sph, 7 int2c2e_cart, 8-9 int2e_ip2, 10-11 int3c2e_ip1,
 * 12-13 int3c2e_ip2, 14-15 int2e_ipip1 (sph, cart); 4, 3 or 2 shell indices per item)
 * with OpenMP over items; item q writes its dense block (all components) at out + offsets[q].
 * Returns wall seconds, or -1 for an unknown kind. */
double oracle_list(int which, const int *items, long n, double *out, const long *offsets,
                   int *atm, int natm, int *bas, int nbas, double *env, int nthreads)
{
    typedef int (*fn_t)(double *, int *, int *, int *, int, int *, int, double *, void *, double *);
    static const fn_t fns[16] = {oracle_int2e_sph, oracle_int2e_cart, oracle_int2e_ip1_sph,
                                 oracle_int2e_ip1_cart, oracle_int3c2e_sph, oracle_int3c2e_cart,
                                 oracle_int2c2e_sph, oracle_int2c2e_cart, oracle_int2e_ip2_sph,
                                 oracle_int2e_ip2_cart, oracle_int3c2e_ip1_sph,
                                 oracle_int3c2e_ip1_cart, oracle_int3c2e_ip2_sph,
                                 oracle_int3c2e_ip2_cart, oracle_int2e_ipip1_sph,
                                 oracle_int2e_ipip1_cart};
    static const int nshs[16] = {4, 4, 4, 4, 3, 3, 2, 2, 4, 4, 3, 3, 3, 3, 4, 4};
    if (which < 0 || which > 15) return -1;
    const int nsh = nshs[which];
    double t0 = 0, t1 = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    t0 = omp_get_wtime();
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (long q = 0; q < n; q++)
        fns[which](out + offsets[q], NULL, (int *)(items + (long)nsh * q), atm, natm, bas, nbas, env,
                   NULL, NULL);
#ifdef _OPENMP
    t1 = omp_get_wtime();
#endif
    return t1 - t0;
}
