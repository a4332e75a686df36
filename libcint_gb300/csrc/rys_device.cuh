/*
 * Device-side building blocks shared by the CUDA translation units of the Rys path
 * (rys_kernels.cu: integrals, J contraction; rys_grad.cu: the adjoint).  Each translation unit
 * that includes this header owns its copy of the small constant tables and fills them through
 * cg_tu_tables_init().
 *
 * Contents: class layout of the per-warp shared memory, Rys node/weight evaluation from the
 * piecewise polynomial tables, Cartesian component powers, and the per-axis vertical recurrence
 * plus both horizontal transfers (libcint CINTg0_2e_2d, src/g2e.c:272-421, and
 * CINTg0_*2d_4d, src/g2e.c:428-693, restated with the i and k centres as bases).
 */
#ifndef CINTGPU_RYS_DEVICE_CUH
#define CINTGPU_RYS_DEVICE_CUH
#include <cuda_runtime.h>
#include <stdint.h>
#include "cintgpu_types.h"
#include "rys_tables.inc"
#include "rys_kernels.h"

#define FULL 0xffffffffu

static __constant__ int c_rys_off[RYS_NMAX + 1];
static __constant__ double c_rys_xmax[RYS_NMAX + 1];
static __constant__ double c_large_r[RYS_NMAX * (RYS_NMAX + 1) / 2];
static __constant__ double c_large_w[RYS_NMAX * (RYS_NMAX + 1) / 2];

/* sparse rows of the cart->sph matrices: row (l, m) has nnz entries (cart index, coefficient) */
#define C2S_MAXNNZ CG_C2S_MAXNNZ
#define C2S_ROWS ((CG_MAX_SHELL_L + 1) * (CG_MAX_SHELL_L + 1))
static __device__ int g_c2s_nnz[C2S_ROWS];
static __device__ int g_c2s_idx[C2S_ROWS * C2S_MAXNNZ];
static __device__ double g_c2s_val[C2S_ROWS * C2S_MAXNNZ];

/* ------------------------------------------------------------------ layout per class */
__host__ __device__ inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

/* Triangle and tetrahedron indexing of Cartesian power tuples: pairs (x, y) with x + y <= L in
 * x-major order, triples (x, y, z) with x + y + z <= L likewise (the contraction-first adjoint
 * keeps its density and contraction arrays in these layouts). */
__host__ __device__ inline int cg_np2(int L) { return L < 0 ? 0 : (L + 1) * (L + 2) / 2; }
__host__ __device__ inline int cg_ntet(int L) { return L < 0 ? 0 : (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ inline int cg_idx2(int L, int x, int y) { return x * (2 * L + 3 - x) / 2 + y; }
__host__ __device__ inline int cg_idx3(int L, int x, int y, int z)
{
    return cg_ntet(L) - cg_ntet(L - x) + cg_idx2(L - x, y, z);
}
__host__ __device__ inline void cg_dec2(int L, int idx, int &x, int &y)
{
    x = 0;
    while (idx > L - x) { idx -= L - x + 1; x++; }
    y = idx;
}
__host__ __device__ inline void cg_dec3(int L, int idx, int &x, int &y, int &z)
{
    x = 0;
    while (idx >= cg_np2(L - x)) { idx -= cg_np2(L - x); x++; }
    cg_dec2(L - x, idx, y, z);
}

/* Per-mode increments of the four g-array axes: derivatives raise the angular momentum the
 * recurrences must reach (ip1: i+1, libcint grad2.c ng = {1,0,0,0,...}; coordinate adjoint:
 * i+1, j+1, k+1; exponent adjoint: +2 on all four). */
__host__ __device__ inline void cg_mode_incs(int mode, int inc[4])
{
    inc[0] = inc[1] = inc[2] = inc[3] = 0;
    if (mode == CG_MODE_IP1) inc[0] = 1;
    else if (mode == CG_MODE_IPIP1) inc[0] = 2;   /* libcint hess.c ng = {2,0,0,0,...} */
    else if (mode == CG_MODE_IP2) inc[2] = 1;   /* libcint grad2.c ng = {0,0,1,0,...} */
    else if (mode == CG_MODE_GRAD) { inc[0] = 1; inc[1] = 1; inc[2] = 1; }
    else if (mode == CG_MODE_GRADA) { inc[0] = 2; inc[1] = 2; inc[2] = 2; inc[3] = 2; }
}

__host__ __device__ inline void cg_class_layout(int li, int lj, int lk, int ll, int mode,
                                                int ws_doubles, CGLayout *L)
{
    int inc[4];
    cg_mode_incs(mode, inc);
    L->lic = li + inc[0];
    L->termw = mode == CG_MODE_GRAD || mode == CG_MODE_GRADA ? CG_TERMW_GRAD : CG_TERMW;
    const int ljc = lj + inc[1], lkc = lk + inc[2], llc = ll + inc[3];
    /* every product the adjoint forms raises ONE center (by 1 for a coordinate, by 2 for an
     * exponent), so the quadrature needs only that much above li+lj+lk+ll even though the g
     * arrays reach the increment on every center */
    const int lsum = li + lj + lk + ll;
    if (mode == CG_MODE_GRAD) L->nroots = (lsum + 1) / 2 + 1;
    else if (mode == CG_MODE_GRADA) L->nroots = (lsum + 2) / 2 + 1;
    else L->nroots = (L->lic + ljc + lkc + llc) / 2 + 1;
    L->nmax = L->lic + ljc;
    L->mmax = lkc + llc;
    L->dI = L->lic + 1; L->dJ = ljc + 1; L->dK = lkc + 1; L->dL = llc + 1;
    L->G = L->dI * L->dJ * L->dK * L->dL;
    L->ng = CG_NG(mode);
    L->nf = ncart(li) * ncart(lj) * ncart(lk) * ncart(ll);
    L->ncomp = CG_NCOMP(mode);
    /* per-lane scratch of g_axis; an odd stride keeps the 32 lanes' equal offsets in distinct
     * shared-memory banks */
    L->scr = (L->nmax + 1) * (L->mmax + 1) + (L->nmax + 1) + (L->mmax + 1);
    L->scr |= 1;
    const bool grad = mode == CG_MODE_GRAD || mode == CG_MODE_GRADA;
    int T = 0;
    if (mode == CG_MODE_GRADJ || mode == CG_MODE_GRADAJ) {
        /* contraction-first adjoint: per term a record (stage-1 values, 2a 2b 2c, m b01; with
         * exponents the term's four primitive indices), the VRR arrays g(e, f) for
         * e <= li+lj+d, f <= lk+ll+d (d = 1, 2 with exponents), and the buffers of one side's
         * axis-by-axis contraction (with exponents also the per-lane exponent partials, 64 per
         * term); per task the transferred densities (bra: also its i-weighted and AB-derivative
         * transfers; ket: its k-weighted transfer), the per-entry sums
         * over terms (three on the bra, two on the ket) and, with exponents, the exponent weights
         * of the four shells and their per-primitive sums */
        const bool ex = mode == CG_MODE_GRADAJ;
        const int Le = li + lj, Lf = lk + ll, d = ex ? 2 : 1;
        L->nroots = (lsum + d) / 2 + 1;
        L->nmax = Le + d;
        L->mmax = Lf + d;
        const int na = L->nmax + 1, nm = L->mmax + 1;
        L->G = na * nm;
        L->gax = L->G | 1;
        L->gstride = 3 * L->gax;
        L->termw = (13 + nm + (ex ? 2 : 0)) | 1;
        const int bufb = cg_np2(Lf) * na + (Lf + 1) * cg_np2(L->nmax);
        const int bufk = cg_np2(Le) * nm + (Le + 1) * cg_np2(L->mmax);
        L->scr = ((bufb > bufk ? bufb : bufk) + (ex ? 64 : 0)) | 1;
        const int tE = cg_ntet(L->nmax), tF = cg_ntet(L->mmax);
        const int fixed = 7 * cg_ntet(Le) + 4 * cg_ntet(Lf) + 3 * tE + 2 * tF
                        + (ex ? 2 * tE + 2 * tF + 4 * CG_GRAD_MAXPRIM : 0);
        T = (ws_doubles - fixed) / (L->termw + L->gstride + L->scr);
        if (T > 32) T = 32;
        if (T < 0) T = 0;
        L->off_dij = L->off_dkl = L->off_aacc = 0;
        L->off_w = fixed;                          /* term records */
        L->off_g = fixed + T * L->termw;
        L->off_scr = L->off_g + T * L->gstride;
    } else if (mode == CG_MODE_ERI) {
        /* contraction first: per term only the VRR arrays g(e, f), e <= li+lj, f <= lk+ll; term
         * records hold the 10 stage-1 values and m b01 for m <= mmax (odd length) */
        L->G = (L->nmax + 1) * (L->mmax + 1);
        L->scr = 0;
        L->gax = L->G | 1;
        L->gstride = 3 * L->gax;
        L->termw = 10 + L->mmax + 1;
        if (L->termw % 2 == 0) L->termw++;
        T = ws_doubles / (L->termw + L->gstride);
        if (T > 32) T = 32;
        if (T < 0) T = 0;
        L->off_dij = L->off_dkl = L->off_aacc = L->off_w = L->off_scr = 0;
        L->off_g = T * L->termw;
    } else if (mode == CG_MODE_ERIB) {
        /* bra transferred per term: per axis g(i, j, f) = out[(i + dI j) + dI dJ f] for i <= li,
         * j <= lj, f <= lk+ll (the VRR array fits inside it, since dI dJ >= li+lj+1); the lane
         * scratch holds one VRR column */
        L->G = L->dI * L->dJ * (L->mmax + 1);
        L->gax = L->G | 1;
        L->gstride = 3 * L->gax;
        L->termw = 10 + L->mmax + 1;
        if (L->termw % 2 == 0) L->termw++;
        L->scr = (L->nmax + 1) | 1;
        for (int t = 32; t >= 1; t--) {
            int items = 3 * t < 32 ? 3 * t : 32;
            if (t * (L->termw + L->gstride) + items * L->scr <= ws_doubles) { T = t; break; }
        }
        L->off_dij = L->off_dkl = L->off_aacc = L->off_w = 0;
        L->off_g = T * L->termw;
        L->off_scr = L->off_g + T * L->gstride;
    } else if (!grad) {
        /* T terms need T term records, T*3*ng*G doubles of g arrays and min(32, 3T) lane
         * scratch areas */
        L->gax = (L->ng * L->G) | 1;
        L->gstride = 3 * L->gax;
        for (int t = 32; t >= 1; t--) {
            int items = 3 * t < 32 ? 3 * t : 32;
            if (t * (CG_TERMW + L->gstride) + items * L->scr <= ws_doubles) { T = t; break; }
        }
        L->off_dij = L->off_dkl = L->off_aacc = L->off_w = L->off_scr = 0;
        L->off_g = T * CG_TERMW;
    } else {
        /* adjoint: term records scale with T; density blocks, exponent sums (GRADA) and the
         * cotangent (nf <= CG_W_SMEM) are per task */
        int d1 = (ncart(li) * ncart(lj) + 1) & ~1, d2 = (ncart(lk) * ncart(ll) + 1) & ~1;
        int aa = mode == CG_MODE_GRADA ? 4 * CG_GRAD_MAXPRIM : 0;
        int wsm = L->nf <= CG_W_SMEM ? ((L->nf + 1) & ~1) : 0;
        int fixed = d1 + d2 + aa + wsm;
        /* odd per-term stride of the g arrays: lanes reading the same offset of different terms
         * hit distinct shared-memory banks */
        L->gax = L->G | 1;
        L->gstride = 3 * L->gax;
        for (int t = 32; t >= 1; t--) {
            int items = 3 * t < 32 ? 3 * t : 32;
            if (t * (CG_TERMW_GRAD + L->gstride) + items * L->scr + fixed <= ws_doubles) { T = t; break; }
        }
        L->off_dij = T * CG_TERMW_GRAD;
        L->off_dkl = L->off_dij + d1;
        L->off_aacc = L->off_dkl + d2;
        L->off_w = L->off_aacc + aa;
        L->off_g = L->off_w + wsm;
        L->off_scr = L->off_g + T * L->gstride;
    }
    L->T = T;
}

/* ------------------------------------------------------------------ roots */
__device__ __forceinline__ void rys_node(int n, double x, int r, const double *__restrict__ coef,
                                         double &s, double &w)
{
    if (x >= c_rys_xmax[n]) {
        double rs = rsqrt(x);
        int o = n * (n - 1) / 2 + r;
        s = c_large_r[o] * (rs * rs);
        w = c_large_w[o] * rs;
    } else {
        int k = (int)x;                      /* interval width 1 */
        double y = 2.0 * (x - (double)k) - 1.0;
        const double2 *c = reinterpret_cast<const double2 *>(
            coef + c_rys_off[n] + (size_t)((k * n + r) * (RYS_DEG + 1)) * 2);
        double2 cj = __ldg(c + RYS_DEG);
        double a = cj.x, b = cj.y;
#pragma unroll
        for (int j = RYS_DEG - 1; j >= 0; j--) {
            cj = __ldg(c + j);
            a = fma(a, y, cj.x);
            b = fma(b, y, cj.y);
        }
        s = a;
        w = b;
    }
}

/* ------------------------------------------------------------------ cart powers */
__device__ __forceinline__ void cart_pow(int l, int p, int &lx, int &ly, int &lz)
{
    /* CINTcart_comp order (src/cint_bas.c:166-181): row = l - lx, q = lz */
    int row = (int)((sqrtf(8.f * p + 1.f) - 1.f) * 0.5f);
    while ((row + 1) * (row + 2) / 2 <= p) row++;
    while (row * (row + 1) / 2 > p) row--;
    int q = p - row * (row + 1) / 2;
    lx = l - row;
    ly = row - q;
    lz = q;
}

/* VRR only (contraction-first path): g(a, m) = out[a + (nmax+1) m] for a <= nmax, m <= mmax,
 * written straight into the term's g array (libcint CINTg0_2e_2d, src/g2e.c:272-330):
 *   g(a+1, 0)   = c00 g(a, 0) + a b10 g(a-1, 0)
 *   g(a, m+1)   = c0p g(a, m) + m b01 g(a, m-1) + a b00 g(a-1, m)
 * computed column by column (a outer), so a b00 is one running sum per column, and m b01 comes
 * from mb[] (computed once per term for the three axes): 3 FP64 operations per entry. */
__device__ __forceinline__ void vrr_axis(int nmax, int mmax, double b00, double b10,
                                         const double *__restrict__ mb, double c00, double c0p,
                                         double g00, double *out)
{
    const int na = nmax + 1;
    out[0] = g00;
    if (mmax > 0) out[na] = c0p * g00;
    for (int m = 1; m < mmax; m++)
        out[(m + 1) * na] = fma(mb[m], out[(m - 1) * na], c0p * out[m * na]);
    double nb = 0.0, ab = b00;       /* (a-1) b10, a b00 */
    for (int a = 1; a <= nmax; a++) {
        double v0 = c00 * out[a - 1];
        if (a >= 2) v0 = fma(nb, out[a - 2], v0);
        out[a] = v0;
        for (int m = 0; m < mmax; m++) {
            double v = fma(ab, out[a - 1 + m * na], c0p * out[a + m * na]);
            if (m > 0) v = fma(mb[m], out[a + (m - 1) * na], v);
            out[a + (m + 1) * na] = v;
        }
        nb += b10;
        ab += b00;
    }
}

/* VRR plus the bra transfer of one axis of one term (the libcint order on the bra,
 * CINTg0_2e_lj2d4d / _il2d4d, src/g2e.c:560-693: (i, j+1) = (i+1, j) + AB (i, j) on every column
 * f of the 2D integrals):  out[(i + dI j) + dI dJ f] for i < dI, j < dJ, f <= mmax.  The VRR
 * array g(a, f) = out[a + (nmax+1) f] is built in place first; columns are then transferred from
 * the highest f down, through the lane's one-column scratch col[nmax+1], so every write lands
 * above the VRR columns still to be read (dI dJ >= nmax + 1). */
__device__ __forceinline__ void vrr_bra_axis(int nmax, int mmax, int dI, int dJ, double b00,
                                             double b10, const double *__restrict__ mb, double c00,
                                             double c0p, double g00, double AB, double *col,
                                             double *out)
{
    const int na = nmax + 1, B = dI * dJ;
    vrr_axis(nmax, mmax, b00, b10, mb, c00, c0p, g00, out);
    for (int m = mmax; m >= 0; m--) {
        const double *v = out + na * m;
        for (int a = 0; a < na; a++) col[a] = v[a];
        double *o = out + B * m;
        for (int i = 0; i < dI; i++) o[i] = col[i];
        for (int j = 1; j < dJ; j++) {
            for (int a = 0; a <= nmax - j; a++) col[a] = fma(AB, col[a], col[a + 1]);
            for (int i = 0; i < dI; i++) o[i + dI * j] = col[i];
        }
    }
}

/* ------------------------------------------------------------------ stage 2 */
/* One Cartesian axis of one term: VRR into T2[a + (nmax+1) m], then the two horizontal
 * transfers; final g[((i dJ + j) dK + k) dL + l] goes to gout.  Lane scratch: T2, and a vector of
 * length mmax+1 (m b01, then the ket transfer).
 * swap bit 0: the bra recurrences run about B = A - AB instead of A (the transfer then builds i
 * from j: (i+1, j) = (i, j+1) + BA (i, j)); bit 1 likewise on the ket.  The planner sets them when
 * the second shell of a pair is the tighter one: the product densities sit near the tighter
 * centre, and moments about the other, distant one make the transfer cancel (a distant,
 * exponent-asymmetric pair loses up to 1e-7 relative that way). */
__device__ __forceinline__ void g_axis(const CGLayout &L, double b00, double b10, double b01,
                                       double c00, double c0p, double g00, double AB, double CD,
                                       double *scr, double *gout, int swap = 0)
{
    const int nmax = L.nmax, mmax = L.mmax, na = nmax + 1, nm = mmax + 1;
    const bool sij = (swap & 1) != 0, skl = (swap & 2) != 0;
    if (sij) { c00 += AB; AB = -AB; }
    if (skl) { c0p += CD; CD = -CD; }
    double *T2 = scr;
    /* m b01 in the vector the transfers use later, then the column-order VRR */
    {
        double *mbv = scr + na * nm + na;
        double mb = 0.0;
        for (int m = 0; m <= mmax; m++) { mbv[m] = mb; mb += b01; }
        vrr_axis(nmax, mmax, b00, b10, mbv, c00, c0p, g00, T2);
    }
    /* (a,0| -> (base, other| one transfer level t at a time, in place on every column m:
     * col[a] = col[a+1] + AB col[a]; after level t, row b of all columns is g(b, t, m) and goes
     * through |m,0) -> |base, other) in a short vector, so no (i,j,m) intermediate is stored. */
    double *tmp = scr + na * nm + na;
    const int nb = sij ? L.dJ : L.dI, nt = sij ? L.dI : L.dJ;     /* bra: base / transfer count */
    const int mb = skl ? L.dL : L.dK, mt = skl ? L.dK : L.dL;     /* ket */
    for (int t = 0; t < nt; t++) {
        if (t > 0) {
            for (int m = 0; m <= mmax; m++) {
                double *col = T2 + m * na;
                for (int a = 0; a <= nmax - t; a++) col[a] = fma(AB, col[a], col[a + 1]);
            }
        }
        for (int b = 0; b < nb; b++) {
            const int i = sij ? t : b, j = sij ? b : t;
            double *go = gout + (i * L.dJ + j) * L.dK * L.dL;
            for (int m = 0; m <= mmax; m++) tmp[m] = T2[b + na * m];
            for (int u = 0; u < mt; u++) {
                if (u > 0)
                    for (int m = 0; m <= mmax - u; m++) tmp[m] = fma(CD, tmp[m], tmp[m + 1]);
                for (int v = 0; v < mb; v++) {
                    const int k = skl ? u : v, l = skl ? v : u;
                    go[k * L.dL + l] = tmp[v];
                }
            }
        }
    }
}


/* components of all shells below l: l (l+1) (l+2) / 6 */
__host__ __device__ __forceinline__ int ncart_below(int l) { return l * (l + 1) * (l + 2) / 6; }

/* Horizontal transfer of one contracted quartet, warp-cooperative (libcint CINTg0_2e_il2d4d /
 * CINTg0_2e_lj2d4d, src/g2e.c:560-693, applied to the contracted (e0|f0) block instead of each
 * primitive's 2D integrals):
 *   (e, j+1_x | = (e+1_x, j| + AB_x (e, j|      on the bra, the lowest non-zero axis of j,
 *   |f, l+1_x)  = |f+1_x, l) + CD_x |f, l)      then on the ket.
 * src holds the accumulators in the class's group layout; prog is the class's transfer program
 * (built on the host: per level the source rows and the axis of every target row).  The
 * Cartesian block comes back in gctr order (i + nfi (k + nfk (l + nfl j))) in h1 or h2 (the
 * returned pointer). */
__device__ inline double *cg_hrr(const double *src, const int *__restrict__ eperm,
                                 const int *__restrict__ fperm, const int *__restrict__ prog,
                                 int li, int lj, int lk, int ll, const double *AB, const double *CD,
                                 double *h1, double *h2, int lane, int bra_done)
{
    /* bra_done: src rows are already (i j| in the order i nfj + j; only the ket levels run */
    const int nE = bra_done ? ncart(li) * ncart(lj) : ncart_below(li + lj + 1) - ncart_below(li);
    const int nF = ncart_below(lk + ll + 1) - ncart_below(lk);
    for (int e = lane; e < nE * nF; e += 32) {
        int ei = e / nF, fi = e - ei * nF;
        h1[e] = src[__ldg(eperm + ei) * nF + __ldg(fperm + fi)];
    }
    __syncwarp();
    double *cur = h1, *nxt = h2;
    const double ab0 = AB[0], ab1 = AB[1], ab2 = AB[2], cd0 = CD[0], cd1 = CD[1], cd2 = CD[2];
    /* bra: level b holds [(ei nc(b) + jb) nF + f] */
    for (int b = 1; b <= (bra_done ? 0 : lj); b++) {
        const int nrows = __ldg(prog);
        const int *rows = prog + 1;
        const double *__restrict__ c = cur;
        double *__restrict__ x = nxt;
        for (int e = lane; e < nrows * nF; e += 32) {
            const int r = e / nF, f = e - r * nF;
            const int hi = __ldg(rows + 3 * r), lo = __ldg(rows + 3 * r + 1), ax = __ldg(rows + 3 * r + 2);
            const double t = ax == 0 ? ab0 : (ax == 1 ? ab1 : ab2);
            x[e] = fma(t, c[lo * nF + f], c[hi * nF + f]);
        }
        prog += 1 + 3 * nrows;
        __syncwarp();
        double *t = cur; cur = nxt; nxt = t;
    }
    /* ket: level d holds [ij out_stride + (fi nc(d) + ld)] */
    const int nfi = ncart(li), nfj = ncart(lj), nfk = ncart(lk), nfl = ncart(ll);
    const int nij = nfi * nfj;
    for (int d = 1; d <= ll; d++) {
        const int nent = __ldg(prog), sin = __ldg(prog + 1), sout = __ldg(prog + 2);
        const int *ents = prog + 3;
        const double *__restrict__ c = cur;
        double *__restrict__ x = nxt;
        for (int e = lane; e < nij * nent; e += 32) {
            const int ij = e / nent, q = e - ij * nent;
            const int hi = __ldg(ents + 3 * q), lo = __ldg(ents + 3 * q + 1), ax = __ldg(ents + 3 * q + 2);
            const double t = ax == 0 ? cd0 : (ax == 1 ? cd1 : cd2);
            x[ij * sout + q] = fma(t, c[ij * sin + lo], c[ij * sin + hi]);
        }
        prog += 3 + 3 * nent;
        __syncwarp();
        double *t = cur; cur = nxt; nxt = t;
    }
    /* cur[((i nfj + j) nfk + k) nfl + l] -> gctr order */
    const int nf = nij * nfk * nfl;
    {
        const double *__restrict__ c = cur;
        double *__restrict__ x = nxt;
        for (int e = lane; e < nf; e += 32) {
            int i = e % nfi, r = e / nfi;
            int k = r % nfk; r /= nfk;
            int l = r % nfl, j = r / nfl;
            x[e] = c[((i * nfj + j) * nfk + k) * nfl + l];
        }
    }
    __syncwarp();
    return nxt;
}

/* fill this translation unit's copies of the tables */
static int cg_tu_tables_init(const int *c2s_nnz, const int *c2s_idx, const double *c2s_val)
{
    double xmax[RYS_NMAX + 1];
    xmax[0] = 0;
    for (int n = 1; n <= RYS_NMAX; n++) xmax[n] = RYS_H * rys_nint_host[n];
    cudaError_t e;
    if ((e = cudaMemcpyToSymbol(c_rys_off, rys_off_host, sizeof(rys_off_host))) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyToSymbol(c_rys_xmax, xmax, sizeof(xmax))) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyToSymbol(c_large_r, rys_large_r_host, sizeof(rys_large_r_host))) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyToSymbol(c_large_w, rys_large_w_host, sizeof(rys_large_w_host))) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyToSymbol(g_c2s_nnz, c2s_nnz, sizeof(int) * C2S_ROWS)) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyToSymbol(g_c2s_idx, c2s_idx, sizeof(int) * C2S_ROWS * C2S_MAXNNZ)) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyToSymbol(g_c2s_val, c2s_val, sizeof(double) * C2S_ROWS * C2S_MAXNNZ)) != cudaSuccess) return (int)e;
    return 0;
}

__device__ __forceinline__ double common_fac_sp(int l)   /* libcint src/g1e.c:565-572 */
{
    return l == 0 ? 0.282094791773878143 : (l == 1 ? 0.488602511902919921 : 1.0);
}

/* Stage 1 for one term (primitive quartet q = kl * nij + ij, root r; short-range plans: 2n terms
 * per primitive quartet, see below): x, prefactor, Rys node and weight, and the division-free recurrence coefficients (libcint CINTg0_2e, src/g2e.c:4425-4545,
 * rewritten in s = t^2: b00 = s / 2(aij+akl), b10 = b00 + (1-s)/2aij, b01 = b00 + (1-s)/2akl,
 * c00 = PA - s akl/(aij+akl) PQ, c0p = QC + s aij/(aij+akl) PQ).  rec[9] = weight * prefactor. */
__device__ __forceinline__ void cg_term(const CGPrimPair &A, const CGPrimPair &B, const CGPair &pij,
                                        const CGPair &pkl, int n, int r, double common,
                                        const double *__restrict__ coef, double *rec,
                                        double omega2 = 0.0, double expcut = 0.0)
{
    double aijkl = A.a + B.a;
    double rs = rsqrt(aijkl);
    double inv = rs * rs;
    double PQx = A.P[0] - B.P[0], PQy = A.P[1] - B.P[1], PQz = A.P[2] - B.P[2];
    double rr = fma(PQx, PQx, fma(PQy, PQy, PQz * PQz));
    double rho = A.a * B.a * inv;
    double x = rho * rr;
    double s, w;
    double fac1 = common * A.K * B.K * rs * A.inv_a * B.inv_a;
    if (omega2 < 0.0) {
        /* short-range Coulomb erfc(omega r)/r, omega^2 = -omega2: the full quadrature (terms
         * r < n) minus the long-range one (terms n <= r < 2n: nodes theta s, weights
         * -sqrt(theta) w at theta x), libcint's two-quadrature form of CINTg0_2e
         * (src/g2e.c:4447-4476) used here for every order; a primitive quartet whose theta x
         * exceeds its screening budget (expcutoff - cce_ij - cce_kl) or 40 is dropped, as libcint
         * does */
        const double theta = -omega2 / (rho - omega2);
        const double tx = theta * x;
        if (r < n) {
            rys_node(n, x, r, coef, s, w);
        } else {
            rys_node(n, tx, r - n, coef, s, w);
            s *= theta;
            fac1 *= -sqrt(theta);
        }
        if (tx > fmin(expcut - A.cce - B.cce, 40.0)) fac1 = 0.0;
    } else if (omega2 > 0.0) {
        /* long-range Coulomb erf(omega r)/r (libcint CINTg0_2e, src/g2e.c:4477-4492): the
         * quadrature of theta x, theta = omega^2 / (omega^2 + rho), weights times sqrt(theta),
         * nodes t^2 -> theta t^2 (in s = t^2 the coefficients below stay linear in s) */
        const double theta = omega2 / (omega2 + rho);
        rys_node(n, x * theta, r, coef, s, w);
        s *= theta;
        fac1 *= sqrt(theta);
    } else {
        rys_node(n, x, r, coef, s, w);
    }
    double tb = s * inv;                 /* 2 b00 */
    double b00 = 0.5 * tb;
    double oms = 1.0 - s;
    double b10 = fma(0.5 * A.inv_a, oms, b00);
    double b01 = fma(0.5 * B.inv_a, oms, b00);
    double ta = tb * B.a, tc = tb * A.a;
    rec[0] = b00; rec[1] = b10; rec[2] = b01;
    rec[3] = fma(-ta, PQx, A.P[0] - pij.A[0]);
    rec[4] = fma(-ta, PQy, A.P[1] - pij.A[1]);
    rec[5] = fma(-ta, PQz, A.P[2] - pij.A[2]);
    rec[6] = fma(tc, PQx, B.P[0] - pkl.A[0]);
    rec[7] = fma(tc, PQy, B.P[1] - pkl.A[1]);
    rec[8] = fma(tc, PQz, B.P[2] - pkl.A[2]);
    rec[9] = w * fac1;
}

#endif
