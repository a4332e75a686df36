/*
 * GB300 (sm_103a) kernels of the Rys-quadrature two-electron integral path.
 *
 * The path is FP64-pipe bound (measured on GB300: 1.2 TFLOP/s DFMA against 74 TFLOP/s FFMA), so
 * the kernels spend FP64 instructions only on the quadrature itself:
 *   - recurrence coefficients are division free (linear in the Rys node s = t^2),
 *   - roots/weights come from piecewise polynomial tables (Horner, 2 x 10 DFMA per root),
 *   - pair quantities (exponential prefactors, product centres) are precomputed once per
 *     primitive pair; libcint's primitive screening (src/cint2e.c:400-425) runs on the host,
 *     which hands each task its list of surviving primitive quartets,
 *   - all index arithmetic is integer.
 *
 * Work decomposition: one warp owns one task (a shell quartet or a slice of its surviving
 * primitive quartets, taken from an atomic counter in longest-first order) and walks its
 * "terms" (primitive quartet x root) 32 at a time:
 *   stage 1   one lane per term: x, prefactor, root, weight and the recurrence coefficients
 *             (libcint CINTg0_2e, src/g2e.c:4425-4545);
 *   stage 2   one lane per (term, Cartesian axis): the 2D vertical recurrence into shared memory
 *             (CINTg0_2e_2d, src/g2e.c:272-421);
 *   stage 3   int2e / int3c2e / J (rys_eri_kernel_e0f0): the contracted (e0|f0) block, one
 *             group (ex, ey, fx, fy) per lane; the horizontal transfer (src/g2e.c:428-693) then
 *             runs once per contracted quartet.
 *             int2e_ip1 and int2e classes with lj or ll >= 4 (rys_eri_kernel_ip1 / _prim):
 *             both transfers per term in stage 2, then one lane per Cartesian component sums
 *             gx gy gz (CINTgout2e, src/cint2e.c:961-1183) or the nabla-i products of int2e_ip1
 *             (src/autocode/grad2.c:19-68).
 * The warp that completes a quartet's last slice sums the slices, transfers, transforms to the
 * requested layout (cart or real spherical, c2s_sph_2e1 / c2s_sph_3c2e1 semantics,
 * src/cart2sph.c:5324-5383, 5884-5925) and stores with arbitrary strides; cg_output_kernel does
 * the same for quartets of plans that keep it separate and zero-fills empty quartets.
 */
#include "rys_device.cuh"

/* piecewise polynomial Rys tables (rys_tables.inc), copied in at initialisation */
static __device__ double g_rys_coef[RYS_NCOEF];

__global__ void rys_roots_kernel(const double *__restrict__ xs, int count, int n,
                                 const double *__restrict__ coef, double *s_out, double *w_out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    for (int r = 0; r < n; r++) {
        double s, w;
        rys_node(n, xs[i], r, coef, s, w);
        s_out[(size_t)i * n + r] = s;
        w_out[(size_t)i * n + r] = w;
    }
}


/* ------------------------------------------------------------------ main kernel */

/* J and K contractions of one slice's Cartesian block (gctr order; linear, so slices contract
 * independently).  Unique quartet (ij|kl) in kernel order, D symmetric:
 *   J (jmode bit 0): X[i,j] += s_kl sum_kl (ij|kl) D[k,l];  X[k,l] += s_ij sum_ij (ij|kl) D[i,j] if
 *       IJ != KL, s = 2 for a pair of two different shells;  J = X + X^T - diag-blocks(X);
 *   K (jmode bit 1): X[i,k] += w sum_jl (ij|kl) D[j,l],  X[j,k] += w sum_il (ij|kl) D[i,l],
 *       X[i,l] += w sum_jk (ij|kl) D[j,k],  X[j,l] += w sum_ik (ij|kl) D[i,k], w halved for each
 *       coincidence (I = J, K = L, IJ = KL): the four transposed pairs of the 8 permutations, each
 *       counted once per distinct permutation;  K = X + X^T. */
__device__ __forceinline__ void cg_k_contract(const CGLaunch &P, const CGTask &tk, const CGPair &pij,
                                              const CGPair &pkl, const double *cart, int lane)
{
    const int nfi = ncart(pij.la), nfj = ncart(pij.lb), nfk = ncart(pkl.la), nfl = ncart(pkl.lb);
    const int nao = P.nao;
    const double w = ((tk.sym & 1) ? 1.0 : 0.5) * ((tk.sym & 2) ? 1.0 : 0.5) * ((tk.sym & 4) ? 1.0 : 0.5);
    const int oi = pij.ao_a, oj = pij.ao_b, ok = pkl.ao_a, ol = pkl.ao_b;
    const double *__restrict__ D = P.dm;
    auto at = [&](int i, int j, int k, int l) { return cart[i + nfi * (k + nfk * (l + nfl * j))]; };
    for (int e = lane; e < nfi * nfk; e += 32) {            /* X[i,k]: D[j,l] */
        const int i = e % nfi, k = e / nfi;
        double v = 0.0;
        for (int j = 0; j < nfj; j++)
            for (int l = 0; l < nfl; l++) v = fma(at(i, j, k, l), __ldg(D + (size_t)(oj + j) * nao + ol + l), v);
        atomicAdd(P.vk + (size_t)(oi + i) * nao + ok + k, w * v);
    }
    for (int e = lane; e < nfj * nfk; e += 32) {            /* X[j,k]: D[i,l] */
        const int j = e % nfj, k = e / nfj;
        double v = 0.0;
        for (int l = 0; l < nfl; l++)
            for (int i = 0; i < nfi; i++) v = fma(at(i, j, k, l), __ldg(D + (size_t)(oi + i) * nao + ol + l), v);
        atomicAdd(P.vk + (size_t)(oj + j) * nao + ok + k, w * v);
    }
    for (int e = lane; e < nfi * nfl; e += 32) {            /* X[i,l]: D[j,k] */
        const int i = e % nfi, l = e / nfi;
        double v = 0.0;
        for (int j = 0; j < nfj; j++)
            for (int k = 0; k < nfk; k++) v = fma(at(i, j, k, l), __ldg(D + (size_t)(oj + j) * nao + ok + k), v);
        atomicAdd(P.vk + (size_t)(oi + i) * nao + ol + l, w * v);
    }
    for (int e = lane; e < nfj * nfl; e += 32) {            /* X[j,l]: D[i,k] */
        const int j = e % nfj, l = e / nfj;
        double v = 0.0;
        for (int k = 0; k < nfk; k++)
            for (int i = 0; i < nfi; i++) v = fma(at(i, j, k, l), __ldg(D + (size_t)(oi + i) * nao + ok + k), v);
        atomicAdd(P.vk + (size_t)(oj + j) * nao + ol + l, w * v);
    }
}

__device__ __forceinline__ void cg_j_contract(const CGLaunch &P, const CGTask &tk, const CGPair &pij,
                                              const CGPair &pkl, const double *cart, int lane)
{
    if (P.jmode & 2) cg_k_contract(P, tk, pij, pkl, cart, lane);
    if (!(P.jmode & 1)) { __syncwarp(); return; }
    const int li = pij.la, lj = pij.lb, lk = pkl.la, ll = pkl.lb;
    const int nfi = ncart(li), nfj = ncart(lj), nfk = ncart(lk), nfl = ncart(ll);
    const int nao = P.nao;
    const double skl = (tk.sym & 2) ? 2.0 : 1.0, sij = (tk.sym & 1) ? 2.0 : 1.0;
    const double *Dkl = P.dm + (size_t)pkl.ao_a * nao + pkl.ao_b;
    for (int e = lane; e < nfi * nfj; e += 32) {
        int i = e % nfi, j = e / nfi;
        double v = 0.0;
        for (int l = 0; l < nfl; l++)
            for (int k = 0; k < nfk; k++)
                v = fma(cart[i + nfi * (k + nfk * (l + nfl * j))], __ldg(Dkl + (size_t)k * nao + l), v);
        atomicAdd(P.vj + (size_t)(pij.ao_a + i) * nao + pij.ao_b + j, skl * v);
    }
    if (tk.sym & 4) {
        const double *Dij = P.dm + (size_t)pij.ao_a * nao + pij.ao_b;
        for (int e = lane; e < nfk * nfl; e += 32) {
            int k = e % nfk, l = e / nfk;
            double v = 0.0;
            for (int j = 0; j < nfj; j++)
                for (int i = 0; i < nfi; i++)
                    v = fma(cart[i + nfi * (k + nfk * (l + nfl * j))], __ldg(Dij + (size_t)i * nao + j), v);
            atomicAdd(P.vj + (size_t)(pkl.ao_a + k) * nao + pkl.ao_b + l, sij * v);
        }
    }
    __syncwarp();
}



/* One task in libcint's order (per primitive: VRR and both transfers, then the products per
 * Cartesian component): int2e_ip1, and int2e classes whose transfers after contraction would
 * amplify rounding beyond 1e-12 (lj or ll >= 4: the 3D transfer multiplies the per-axis
 * amplifications that libcint's per-axis transfers only add).
 * NS > 0: lane-private register accumulators for components c = lane + 32 s, s < NS
 * NS = 0: accumulators in the task's slot (large classes). */
template <int MODE, int NS>
__device__ __forceinline__ void run_task(const CGLaunch &P, const CGTask &tk, const CGLayout &L,
                                         double *term, double *greg, int lane)
{
    const CGPair pij = P.pairs[tk.pij];
    const CGPair pkl = P.pairs[tk.pkl];
    const CGPrimPair *__restrict__ ppij = P.prims + pij.prim_off;
    const CGPrimPair *__restrict__ ppkl = P.prims + pkl.prim_off;
    const int *__restrict__ pql = P.pqlist + tk.pq_off;
    const int nij = pij.npa * pij.npb;
    const int li = pij.la, lj = pij.lb, lk = pkl.la, ll = pkl.lb;
    const int nfi = ncart(li), nfj = ncart(lj), nfk = ncart(lk), nfl = ncart(ll);
    const int n = L.nroots;
    const int T = L.T;
    const double common = P.common_base * common_fac_sp(li) * (P.two ? 1.0 : common_fac_sp(lj))
                        * common_fac_sp(lk) * (P.three ? 1.0 : common_fac_sp(ll));
    double *scr_base = greg + T * L.gstride;
    double *acc = P.jmode ? P.wscratch + (size_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * P.wscratch_stride
                          : P.gctr + tk.cart_off;

    /* per-lane component offsets into the g arrays (register path: packed 10 bits per axis, G < 1024) */
    int offs[NS > 0 ? NS : 1];
    /* accumulators per component: 1; 3 nabla components; 6 distinct second-nabla components
     * (xx, yy, zz, xy, xz, yz) */
    constexpr int NACC = MODE == CG_MODE_IPIP1 ? 6 : (CG_IS_IP(MODE) ? 3 : 1);
    double ra[NS > 0 ? NS : 1][NACC];
    auto comp_offsets3 = [&](int c, int &ox, int &oy, int &oz) {
        int ic = c % nfi, rest = c / nfi;
        int kc = rest % nfk; rest /= nfk;
        int lc = rest % nfl;
        int jc = rest / nfl;
        int ix, iy, iz, jx, jy, jz, kx, ky, kz, lx, ly, lz;
        cart_pow(li, ic, ix, iy, iz);
        cart_pow(lj, jc, jx, jy, jz);
        cart_pow(lk, kc, kx, ky, kz);
        cart_pow(ll, lc, lx, ly, lz);
        ox = ((ix * L.dJ + jx) * L.dK + kx) * L.dL + lx;
        oy = ((iy * L.dJ + jy) * L.dK + ky) * L.dL + ly;
        oz = ((iz * L.dJ + jz) * L.dK + kz) * L.dL + lz;
    };
    auto comp_offsets = [&](int c) -> int {
        int ox, oy, oz;
        comp_offsets3(c, ox, oy, oz);
        return ox | (oy << 10) | (oz << 20);
    };
    if (NS > 0) {
#pragma unroll
        for (int s = 0; s < (NS > 0 ? NS : 1); s++) {
            int c = lane + 32 * s;
            offs[s] = c < L.nf ? comp_offsets(c) : 0;
#pragma unroll
            for (int q = 0; q < NACC; q++) ra[s][q] = 0.0;
        }
    } else {
        for (int c = lane; c < L.nf * L.ncomp; c += 32) acc[c] = 0.0;
    }

    const int nt = P.omega2 < 0.0 ? 2 * n : n;   /* terms per primitive quartet */
    const int nterm = tk.npq * nt;
    for (int t0 = 0; t0 < nterm; t0 += T) {
        const int Tb = min(T, nterm - t0);
        /* ---- stage 1: one lane per term */
        if (lane < Tb) {
            int g = t0 + lane;
            int p = g / nt, r = g - p * nt;
            int q = __ldg(pql + p);
            int kl = q / nij, ij = q - kl * nij;
            const CGPrimPair A = ppij[ij];
            const CGPrimPair B = ppkl[kl];
            double *rec = term + lane * CG_TERMW;
            cg_term(A, B, pij, pkl, n, r, common, P.rys_coef, rec, P.omega2, P.expcut);
            rec[10] = -2.0 * (MODE == CG_MODE_IP2 ? B.aA : A.aA);   /* -2 a of the nabla shell */
        }
        __syncwarp();
        /* ---- stage 2: one lane per (term, axis) */
        for (int item = lane; item < 3 * Tb; item += 32) {
            int t = item / 3, ax = item - 3 * t;
            const double *rec = term + t * CG_TERMW;
            double g00 = (ax == 2) ? rec[9] : 1.0;
            double *gdst = greg + (size_t)(t * 3 + ax) * L.gax;
            g_axis(L, rec[0], rec[1], rec[2], rec[3 + ax], rec[6 + ax], g00,
                   pij.AB[ax], pkl.AB[ax], scr_base + lane * L.scr, gdst, (tk.sym >> 3) & 3);
            if (MODE == CG_MODE_IP1 || MODE == CG_MODE_IPIP1) {
                /* f(i) = i g(i-1) - 2 a_i g(i+1)   (CINTnabla1i_2e, src/g2e.c:4550-4591); with two
                 * nablas the same once more on f: h(i) = i f(i-1) - 2 a_i f(i+1) */
                const double ai2 = rec[10];
                const int sI = L.dJ * L.dK * L.dL;
                for (int pass = 0; pass < (MODE == CG_MODE_IPIP1 ? 2 : 1); pass++) {
                    const double *g = gdst + pass * L.G;
                    double *f = gdst + (pass + 1) * L.G;
                    for (int i = 0; i < L.dI - 1 - pass; i++) {
                        for (int o = 0; o < sI; o++) {
                            double v = ai2 * g[(i + 1) * sI + o];
                            if (i > 0) v = fma((double)i, g[(i - 1) * sI + o], v);
                            f[i * sI + o] = v;
                        }
                    }
                }
            } else if (MODE == CG_MODE_IP2) {
                /* f(k) = k g(k-1) - 2 a_k g(k+1) along k (CINTnabla1k_2e, src/g2e.c:4651-4701) */
                const double ak2 = rec[10];
                const int dK = L.dK, dL = L.dL, nij = L.dI * L.dJ;
                double *f = gdst + L.G;
                for (int ij = 0; ij < nij; ij++) {
                    const double *g0 = gdst + ij * dK * dL;
                    double *f0 = f + ij * dK * dL;
                    for (int k = 0; k < dK - 1; k++)
                        for (int l = 0; l < dL; l++) {
                            double v = ak2 * g0[(k + 1) * dL + l];
                            if (k > 0) v = fma((double)k, g0[(k - 1) * dL + l], v);
                            f0[k * dL + l] = v;
                        }
                }
            }
        }
        __syncwarp();
        /* ---- stage 3: one lane per Cartesian component */
        const int stride_t = L.gstride;
        const int G = L.G, A = L.gax;   /* f arrays at +G inside an axis block; axis blocks A apart */
        if (NS > 0) {
#pragma unroll
            for (int s = 0; s < (NS > 0 ? NS : 1); s++) {
                if (lane + 32 * s >= L.nf) continue;
                const int ox = offs[s] & 1023, oy = (offs[s] >> 10) & 1023, oz = offs[s] >> 20;
                const double *gb = greg;
                if (MODE == CG_MODE_IPIP1) {
                    double a[6];
#pragma unroll
                    for (int q = 0; q < 6; q++) a[q] = ra[s][q < NACC ? q : 0];
                    for (int t = 0; t < Tb; t++, gb += stride_t) {
                        const double gx = gb[ox], gy = gb[A + oy], gz = gb[2 * A + oz];
                        const double fx = gb[G + ox], fy = gb[A + G + oy], fz = gb[2 * A + G + oz];
                        const double hx = gb[2 * G + ox], hy = gb[A + 2 * G + oy], hz = gb[2 * A + 2 * G + oz];
                        a[0] = fma(hx, gy * gz, a[0]);
                        a[1] = fma(hy, gx * gz, a[1]);
                        a[2] = fma(hz, gx * gy, a[2]);
                        a[3] = fma(fx * fy, gz, a[3]);
                        a[4] = fma(fx * fz, gy, a[4]);
                        a[5] = fma(fy * fz, gx, a[5]);
                    }
#pragma unroll
                    for (int q = 0; q < 6; q++) ra[s][q < NACC ? q : 0] = a[q];
                } else if (CG_IS_IP(MODE)) {
                    double sx = ra[s][0], sy = ra[s][CG_IS_IP(MODE) ? 1 : 0],
                           sz = ra[s][CG_IS_IP(MODE) ? 2 : 0];
                    for (int t = 0; t < Tb; t++, gb += stride_t) {
                        double gx = gb[ox], gy = gb[A + oy], gz = gb[2 * A + oz];
                        double fx = gb[G + ox], fy = gb[A + G + oy], fz = gb[2 * A + G + oz];
                        sx = fma(fx, gy * gz, sx);
                        sy = fma(fy, gx * gz, sy);
                        sz = fma(fz, gx * gy, sz);
                    }
                    ra[s][0] = sx;
                    ra[s][CG_IS_IP(MODE) ? 1 : 0] = sy;
                    ra[s][CG_IS_IP(MODE) ? 2 : 0] = sz;
                } else {
                    double s0 = ra[s][0];
                    for (int t = 0; t < Tb; t++, gb += stride_t)
                        s0 = fma(gb[ox] * gb[A + oy], gb[2 * A + oz], s0);
                    ra[s][0] = s0;
                }
            }
        } else {
            for (int c = lane; c < L.nf; c += 32) {
                int ox, oy, oz;
                comp_offsets3(c, ox, oy, oz);
                const double *gb = greg;
                if (MODE == CG_MODE_IPIP1) {
                    /* components 3a + b; xx, yy, zz, xy, xz, yz here, the mirrors at task end */
                    const int nf = L.nf;
                    double a0 = acc[c], a1 = acc[4 * nf + c], a2 = acc[8 * nf + c];
                    double a3 = acc[nf + c], a4 = acc[2 * nf + c], a5 = acc[5 * nf + c];
                    for (int t = 0; t < Tb; t++, gb += stride_t) {
                        const double gx = gb[ox], gy = gb[A + oy], gz = gb[2 * A + oz];
                        const double fx = gb[G + ox], fy = gb[A + G + oy], fz = gb[2 * A + G + oz];
                        const double hx = gb[2 * G + ox], hy = gb[A + 2 * G + oy], hz = gb[2 * A + 2 * G + oz];
                        a0 = fma(hx, gy * gz, a0);
                        a1 = fma(hy, gx * gz, a1);
                        a2 = fma(hz, gx * gy, a2);
                        a3 = fma(fx * fy, gz, a3);
                        a4 = fma(fx * fz, gy, a4);
                        a5 = fma(fy * fz, gx, a5);
                    }
                    acc[c] = a0; acc[4 * nf + c] = a1; acc[8 * nf + c] = a2;
                    acc[nf + c] = a3; acc[2 * nf + c] = a4; acc[5 * nf + c] = a5;
                } else if (CG_IS_IP(MODE)) {
                    double sx = acc[c], sy = acc[L.nf + c], sz = acc[2 * L.nf + c];
                    for (int t = 0; t < Tb; t++, gb += stride_t) {
                        double gx = gb[ox], gy = gb[A + oy], gz = gb[2 * A + oz];
                        double fx = gb[G + ox], fy = gb[A + G + oy], fz = gb[2 * A + G + oz];
                        sx = fma(fx, gy * gz, sx);
                        sy = fma(fy, gx * gz, sy);
                        sz = fma(fz, gx * gy, sz);
                    }
                    acc[c] = sx; acc[L.nf + c] = sy; acc[2 * L.nf + c] = sz;
                } else {
                    double s0 = acc[c];
                    for (int t = 0; t < Tb; t++, gb += stride_t)
                        s0 = fma(gb[ox] * gb[A + oy], gb[2 * A + oz], s0);
                    acc[c] = s0;
                }
            }
        }
        __syncwarp();
    }
    if (NS > 0) {
#pragma unroll
        for (int s = 0; s < (NS > 0 ? NS : 1); s++) {
            int c = lane + 32 * s;
            if (c < L.nf) {
                if (MODE == CG_MODE_IPIP1) {
                    /* component 3a + b of the symmetric second nabla */
                    const int from[9] = {0, 3, 4, 3, 1, 5, 4, 5, 2};
#pragma unroll
                    for (int q = 0; q < 9; q++) acc[q * L.nf + c] = ra[s][from[q] < NACC ? from[q] : 0];
                } else {
#pragma unroll
                    for (int q = 0; q < NACC; q++) acc[q * L.nf + c] = ra[s][q];
                }
            }
        }
    } else if (MODE == CG_MODE_IPIP1) {
        for (int c = lane; c < L.nf; c += 32) {
            acc[3 * L.nf + c] = acc[L.nf + c];
            acc[6 * L.nf + c] = acc[2 * L.nf + c];
            acc[7 * L.nf + c] = acc[5 * L.nf + c];
        }
    }
    if (MODE == CG_MODE_ERIP && P.jmode) {
        __syncwarp();
        cg_j_contract(P, tk, pij, pkl, acc, lane);
    } else if (lane == 0) {
        P.nonempty[tk.out] = 1;
    }
}

/* ------------------------------------------------------------------ output transform */
/* One warp, one contracted quartet: sum its slices, run the class's horizontal transfer (int2e /
 * int3c2e accumulators), transform j, l, k, i to real spherical harmonics (c2s_sph_2e1 /
 * c2s_sph_3c2e1 semantics, src/cart2sph.c:5324-5383, 5884-5925) and store with the task's strides;
 * an empty quartet is zero-filled (c2s_dset0).  Scratch per warp: s1, s2 (nf_max each), then two
 * transfer buffers sharing the rest of spw.  peer_slots: slices were written by other warps of the
 * running kernel, so they are read past L1. */
__device__ __forceinline__ void c2s_pass(const double *__restrict__ src, double *__restrict__ dst,
                                         int lsh, int sph, int inner, int ncart_t, int outer, int lane)
{
    /* src[(a, t, b)] with a < inner, t < ncart_t, b < outer  ->  dst[(a, m, b)] */
    int nm = sph ? (lsh <= 1 ? ncart_t : 2 * lsh + 1) : ncart_t;
    int total = inner * nm * outer;
    for (int e = lane; e < total; e += 32) {
        int a = e % inner, rest = e / inner;
        int m = rest % nm, b = rest / nm;
        double v;
        if (!sph || lsh <= 1) {
            v = src[(size_t)(b * ncart_t + m) * inner + a];
        } else {
            int row = lsh * lsh + m;     /* rows of l start at l^2 (sum of 2l'+1 for l' < l) */
            int nnz = g_c2s_nnz[row];
            v = 0.0;
            for (int z = 0; z < nnz; z++) {
                v = fma(g_c2s_val[row * C2S_MAXNNZ + z],
                        src[(size_t)(b * ncart_t + g_c2s_idx[row * C2S_MAXNNZ + z]) * inner + a], v);
            }
        }
        dst[(size_t)(b * nm + m) * inner + a] = v;
    }
}

__device__ inline void cg_out_quartet(const CGOutTask &o, bool ne, bool peer_slots, double *gctr,
                                      const CGEriClass *__restrict__ eclass,
                                      const int *__restrict__ eperm, const int *__restrict__ hprog,
                                      double *out, int ncomp, int64_t comp_stride, double *s1,
                                      int64_t nf_max, int64_t spw, int lane, double *own = nullptr)
{
    double *s2 = s1 + nf_max;
    double *h1 = s2 + nf_max;
    double *h2 = h1 + (spw - 2 * nf_max) / 2;
    const int sph = o.flags & 1;
    int nfc[4], nd[4];
    for (int a = 0; a < 4; a++) {
        nfc[a] = ncart(o.l[a]);
        nd[a] = sph ? (o.l[a] <= 1 ? nfc[a] : 2 * o.l[a] + 1) : nfc[a];
    }
    const int nf = nfc[0] * nfc[1] * nfc[2] * nfc[3];
    const bool e0f0 = (o.flags & 2) != 0;
    CGEriClass ec;
    memset(&ec, 0, sizeof(ec));
    if (e0f0) ec = eclass[o.ecls];
    const int slot = e0f0 ? ec.nE * ec.nF : nf;   /* accumulators per part and component */
    for (int comp = 0; comp < ncomp; comp++) {
        /* own: the quartet's single slice sits in this warp's own slot */
        double *g0 = (own ? own : gctr + o.cart_off) + (size_t)comp * slot;
        if (ne && o.nparts > 1) {
            for (int c = lane; c < slot; c += 32) {
                double v = peer_slots ? __ldcg(g0 + c) : g0[c];
                for (int p = 1; p < o.nparts; p++) {
                    const double *gp = g0 + (size_t)p * ncomp * slot + c;
                    v += peer_slots ? __ldcg(gp) : *gp;
                }
                g0[c] = v;
            }
            __syncwarp();
        }
        double *dst = out + o.out_off + (size_t)comp * comp_stride;
        if (!ne) {
            int tot = nd[0] * nd[1] * nd[2] * nd[3];
            for (int e = lane; e < tot; e += 32) {
                int i = e % nd[0], r = e / nd[0];
                int j = r % nd[1]; r /= nd[1];
                int k = r % nd[2], l = r / nd[2];
                dst[(int64_t)i * o.st[0] + (int64_t)j * o.st[1] + (int64_t)k * o.st[2]
                    + (int64_t)l * o.st[3]] = 0.0;
            }
            continue;
        }
        /* a single slice written by another warp: read it past L1 through the transfer's gather */
        if (peer_slots && o.nparts == 1 && !own) {
            for (int c = lane; c < slot; c += 32) g0[c] = __ldcg(g0 + c);
            __syncwarp();
        }
        /* gctr order: i fastest, then k, l, j.  Pass j: inner = nfi*nfk*nfl, t = j */
        const double *cur = g0;
        if (e0f0)
            cur = cg_hrr(g0, eperm + ec.perm_off, eperm + ec.perm_off + ec.nE,
                         hprog + ec.hprog_off, o.l[0], o.l[1], o.l[2], o.l[3], o.AB, o.CD,
                         h1, h2, lane, ec.bra);
        /* a pass on an s or p shell (or any Cartesian one) maps every element to the same index,
         * so it is skipped and the next pass reads its input where it is */
        auto pass = [&](const double *src, int lsh, int inner, int nct, int outer) -> const double * {
            if (!sph || lsh <= 1) return src;
            double *d = src == s1 ? s2 : s1;
            c2s_pass(src, d, lsh, sph, inner, nct, outer, lane);
            __syncwarp();
            return d;
        };
        cur = pass(cur, o.l[1], nfc[0] * nfc[2] * nfc[3], nfc[1], 1);
        /* pass l: (i,k | l | js) */
        cur = pass(cur, o.l[3], nfc[0] * nfc[2], nfc[3], nd[1]);
        /* pass k: (i | k | ls, js) */
        cur = pass(cur, o.l[2], nfc[0], nfc[2], nd[3] * nd[1]);
        /* pass i: (1 | i | ks, ls, js) */
        cur = pass(cur, o.l[0], 1, nfc[0], nd[2] * nd[3] * nd[1]);
        /* layout: (is, ks, ls, js) */
        int tot = nd[0] * nd[2] * nd[3] * nd[1];
        for (int e = lane; e < tot; e += 32) {
            int i = e % nd[0], r = e / nd[0];
            int k = r % nd[2]; r /= nd[2];
            int l = r % nd[3], j = r / nd[3];
            dst[(int64_t)i * o.st[0] + (int64_t)j * o.st[1] + (int64_t)k * o.st[2]
                + (int64_t)l * o.st[3]] = cur[e];
        }
        __syncwarp();
    }
}

/* ---------------------------------------------------------- contraction-first int2e path */
/* Stage 3 of one group over terms t_begin, t_begin + tstep, ... < Tb: p = gx gy once, then
 * r[b * 4 + a] += p gz(ez0 + a, fz0 + b) for the group's nez x nfz members (MA x MB bound). */
template <int MA, int MB>
__device__ __forceinline__ void e0f0_terms(const double *__restrict__ greg, int gstride, int G,
                                           int na, int t_begin, int Tb, int tstep, int oxy,
                                           int oz, int mn, double (&r)[16])
{
    const int ox = oxy & 0xffff, oy = oxy >> 16;
    const int nez = mn & 0xff, nfz = (mn >> 8) & 0xff;
    for (int t = t_begin; t < Tb; t += tstep) {
        const double *g = greg + (size_t)t * gstride;
        const double p = g[ox] * g[G + oy];
        const double *gz = g + 2 * G + oz;
#pragma unroll
        for (int b = 0; b < MB; b++)
#pragma unroll
            for (int a = 0; a < MA; a++)
                if (a < nez && b < nfz) r[b * 4 + a] = fma(p, gz[a + na * b], r[b * 4 + a]);
    }
}

__device__ __forceinline__ void e0f0_dispatch(int mab, const double *greg, int gstride, int G,
                                              int na, int t_begin, int Tb, int tstep, int oxy,
                                              int oz, int mn, double (&r)[16])
{
#define CG_E0F0_CASE(A, B) \
    case (A - 1) + 4 * (B - 1): e0f0_terms<A, B>(greg, gstride, G, na, t_begin, Tb, tstep, oxy, oz, mn, r); break;
    switch (mab) {
    CG_E0F0_CASE(1, 1) CG_E0F0_CASE(2, 1) CG_E0F0_CASE(3, 1) CG_E0F0_CASE(4, 1)
    CG_E0F0_CASE(1, 2) CG_E0F0_CASE(2, 2) CG_E0F0_CASE(3, 2) CG_E0F0_CASE(4, 2)
    CG_E0F0_CASE(1, 3) CG_E0F0_CASE(2, 3) CG_E0F0_CASE(3, 3) CG_E0F0_CASE(4, 3)
    CG_E0F0_CASE(1, 4) CG_E0F0_CASE(2, 4) CG_E0F0_CASE(3, 4) CG_E0F0_CASE(4, 4)
    default: break;
    }
#undef CG_E0F0_CASE
}

/* One int2e / int3c2e / J task, contraction first: per term the VRR arrays only; stage 3
 * accumulates (e0|f0) of the task's slice; the horizontal transfer runs in the output kernel
 * (once per contracted quartet) or, for J, at the end of the task.  Classes with ec.bra (layout
 * CG_MODE_ERIB) transfer the bra per term in stage 2 and accumulate (ij|f0) instead. */
__device__ __forceinline__ void run_task_e0f0(const CGLaunch &P, const CGTask &tk, const CGLayout &L,
                                              double *term, double *greg, int lane)
{
    const CGPair pij = P.pairs[tk.pij];
    const CGPair pkl = P.pairs[tk.pkl];
    const CGPrimPair *__restrict__ ppij = P.prims + pij.prim_off;
    const CGPrimPair *__restrict__ ppkl = P.prims + pkl.prim_off;
    const int *__restrict__ pql = P.pqlist + tk.pq_off;
    const int nij = pij.npa * pij.npb;
    const int li = pij.la, lj = pij.lb, lk = pkl.la, ll = pkl.lb;
    const CGEriClass ec = P.eclass[tk.cls];
    /* G: axis stride; na: stride between the f members of a group (f's step in the axis array) */
    const int n = L.nroots, T = L.T, G = L.gax, gstride = L.gstride;
    const int na = ec.bra ? L.dI * L.dJ : L.nmax + 1;
    const double common = P.common_base * common_fac_sp(li) * (P.two ? 1.0 : common_fac_sp(lj))
                        * common_fac_sp(lk) * (P.three ? 1.0 : common_fac_sp(ll));
    const CGEriGroup *__restrict__ grp = P.egroup + ec.group_off;
    const int nF = ec.nF, nEF = ec.nE * ec.nF;
    double *wbase = P.jmode ? P.wscratch + (size_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * P.wscratch_stride
                            : nullptr;
    double *acc = P.jmode ? wbase
                : tk.own_slot ? P.wslot + (size_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * P.wslot_stride
                              : P.gctr + tk.cart_off;
    const int MA = ec.maxab & 0xff, MB = ec.maxab >> 8;
    const bool boxed = MA <= 4 && MB <= 4;
    const int mab = (MA - 1) + 4 * (MB - 1);
    const int S = ec.split;

    double r[16];
#pragma unroll
    for (int m = 0; m < 16; m++) r[m] = 0.0;
    int sp = 0;
    bool own = false;
    CGEriGroup mine = {0, 0, 0, 0};
    if (S > 0) {
        /* lane = group + ngroup * split: one group per lane for the whole task */
        const int gi = lane % ec.ngroup;
        sp = lane / ec.ngroup;
        own = sp < S;
        if (own) mine = grp[gi];
    } else {
        for (int c = lane; c < nEF; c += 32) acc[c] = 0.0;
        __syncwarp();
    }

    const int nt = P.omega2 < 0.0 ? 2 * n : n;   /* terms per primitive quartet */
    const int nterm = tk.npq * nt;
    for (int t0 = 0; t0 < nterm; t0 += T) {
        const int Tb = min(T, nterm - t0);
        /* ---- stage 1: one lane per term */
        if (lane < Tb) {
            int g = t0 + lane;
            int p = g / nt, rr = g - p * nt;
            int q = __ldg(pql + p);
            int kl = q / nij, ij = q - kl * nij;
            double *rec = term + lane * L.termw;
            cg_term(ppij[ij], ppkl[kl], pij, pkl, n, rr, common, P.rys_coef, rec, P.omega2, P.expcut);
            double mb = 0.0;
            for (int m = 0; m <= L.mmax; m++) { rec[10 + m] = mb; mb += rec[2]; }   /* m b01 */
        }
        __syncwarp();
        /* ---- stage 2: one lane per (term, axis), VRR only (bra classes: and the bra transfer) */
        for (int item = lane; item < 3 * Tb; item += 32) {
            int t = item / 3, ax = item - 3 * t;
            const double *rec = term + t * L.termw;
            double g00 = (ax == 2) ? rec[9] : 1.0;
            if (ec.bra)
                vrr_bra_axis(L.nmax, L.mmax, L.dI, L.dJ, rec[0], rec[1], rec + 10, rec[3 + ax],
                             rec[6 + ax], g00, pij.AB[ax], greg + (size_t)T * gstride + lane * L.scr,
                             greg + (size_t)t * gstride + ax * G);
            else
                vrr_axis(L.nmax, L.mmax, rec[0], rec[1], rec + 10, rec[3 + ax], rec[6 + ax], g00,
                         greg + (size_t)t * gstride + ax * G);
        }
        __syncwarp();
        /* ---- stage 3: groups */
        if (S > 0) {
            if (own) e0f0_dispatch(mab, greg, gstride, G, na, sp, Tb, S, mine.oxy, mine.oz, mine.mn, r);
        } else if (boxed) {
            /* the class's rounds (<= 32 groups, one per lane), each dispatched on its member box */
            for (int ri = 0; ri < ec.nround; ri++) {
                const int rd = __ldg(P.eround + ec.round_off + ri);
                if (lane >= (int)(((unsigned)rd >> 16) & 0xffu)) continue;
                const CGEriGroup q = grp[(rd & 0xffff) + lane];
                const int nez = q.mn & 0xff, nfz = (q.mn >> 8) & 0xff;
                double v[16];
#pragma unroll
                for (int b = 0; b < 4; b++)
#pragma unroll
                    for (int a = 0; a < 4; a++)
                        v[b * 4 + a] = (a < nez && b < nfz) ? acc[q.acc + a * nF + b] : 0.0;
                e0f0_dispatch((int)((unsigned)rd >> 24), greg, gstride, G, na, 0, Tb, 1, q.oxy, q.oz, q.mn, v);
#pragma unroll
                for (int b = 0; b < 4; b++)
#pragma unroll
                    for (int a = 0; a < 4; a++)
                        if (a < nez && b < nfz) acc[q.acc + a * nF + b] = v[b * 4 + a];
            }
        } else {
            /* member at a time (lj or ll above 3) */
            for (int gi = lane; gi < ec.ngroup; gi += 32) {
                const CGEriGroup q = grp[gi];
                const int ox = q.oxy & 0xffff, oy = q.oxy >> 16;
                const int nez = q.mn & 0xff, nfz = (q.mn >> 8) & 0xff;
                for (int b = 0; b < nfz; b++)
                    for (int a = 0; a < nez; a++) {
                        double s0 = acc[q.acc + a * nF + b];
                        const double *g = greg;
                        for (int t = 0; t < Tb; t++, g += gstride)
                            s0 = fma(g[ox] * g[G + oy], g[2 * G + q.oz + a + na * b], s0);
                        acc[q.acc + a * nF + b] = s0;
                    }
            }
        }
        __syncwarp();
    }
    if (S > 0) {
        /* sum the splits (lanes gi + ngroup * sp), then the first split stores its members */
        for (int off = S >> 1; off >= 1; off >>= 1) {
#pragma unroll
            for (int m = 0; m < 16; m++) r[m] += __shfl_down_sync(FULL, r[m], off * ec.ngroup);
        }
        if (own && sp == 0) {
            const int nez = mine.mn & 0xff, nfz = (mine.mn >> 8) & 0xff;
#pragma unroll
            for (int b = 0; b < 4; b++)
#pragma unroll
                for (int a = 0; a < 4; a++)
                    if (a < nez && b < nfz) acc[mine.acc + a * nF + b] = r[b * 4 + a];
        }
        __syncwarp();
    }
    if (P.jmode) {
        /* J contraction of this slice's transferred block */
        const double *cart = cg_hrr(acc, P.eperm + ec.perm_off, P.eperm + ec.perm_off + ec.nE,
                                    P.hprog + ec.hprog_off, li, lj, lk, ll, pij.AB, pkl.AB,
                                    wbase + P.hrr_off1, wbase + P.hrr_off2, lane, ec.bra);
        cg_j_contract(P, tk, pij, pkl, cart, lane);
    } else if (lane == 0) {
        P.nonempty[tk.out] = 1;
    }
}

template <int MODE>
__device__ __forceinline__ void rys_eri_body(const CGLaunch &P)
{
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    double *ws = smem + (size_t)warp * P.ws_doubles;
    double *term = ws;                                   /* term records, then g arrays at L.off_g */

    for (;;) {
        int tid = 0;
        if (lane == 0) tid = atomicAdd(P.counter, 1);
        tid = __shfl_sync(FULL, tid, 0);
        if (tid >= P.ntasks) break;
        const CGTask tk = P.tasks[P.task0 + tid];
        const int la = P.pairs[tk.pij].la, lb = P.pairs[tk.pij].lb;
        const int lc = P.pairs[tk.pkl].la, ld = P.pairs[tk.pkl].lb;
        CGLayout L;
        const int lmode = (MODE == CG_MODE_ERI && P.eclass[tk.cls].bra) ? CG_MODE_ERIB : MODE;
        cg_class_layout(la, lb, lc, ld, lmode, P.ws_doubles, &L);
        const int ns = (L.nf + 31) >> 5;
        if (L.T < 1) {
            if (lane == 0) atomicOr(P.status, 1);
            continue;
        }
        if (MODE == CG_MODE_ERI) run_task_e0f0(P, tk, L, term, ws + L.off_g, lane);
        else if (L.G >= 1024) run_task<MODE, 0>(P, tk, L, term, ws + L.off_g, lane);
        else if (ns <= 1) run_task<MODE, 1>(P, tk, L, term, ws + L.off_g, lane);
        else if (ns <= 4) run_task<MODE, 4>(P, tk, L, term, ws + L.off_g, lane);
        else if (ns <= 16 && MODE == CG_MODE_ERIP) run_task<MODE, 16>(P, tk, L, term, ws + L.off_g, lane);
        else run_task<MODE, 0>(P, tk, L, term, ws + L.off_g, lane);
        if (P.fuse_out) {
            /* publish this slice; the warp completing the quartet's last slice transforms it
             * (every lane fences its slot writes, the warp syncs, then lane 0 counts; the reader
             * fences after the count and reads past L1) */
            __threadfence();
            __syncwarp();
            int last = 0;
            if (lane == 0) last = atomicAdd(P.done + tk.out, 1) == P.outs[tk.out].nparts - 1;
            last = __shfl_sync(FULL, last, 0);
            if (last) {
                __threadfence();
                const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
                cg_out_quartet(P.outs[tk.out], true, true, P.gctr, P.eclass, P.eperm, P.hprog, P.out,
                               P.ncomp, P.comp_stride, P.oscr + (size_t)gw * P.oscr_stride, P.nf_max,
                               P.oscr_stride, lane,
                               tk.own_slot ? P.wslot + (size_t)gw * P.wslot_stride : nullptr);
            }
        }
    }
}

/* int2e / int3c2e / J: the register allocation ptxas picks under the plain bound measured fastest;
 * int2e_ip1 and per-primitive int2e: two CTAs per SM (what shared memory allows anyway) lets them
 * keep every value in registers instead of spilling */
__global__ void __launch_bounds__(128) rys_eri_kernel_e0f0(CGLaunch P) { rys_eri_body<CG_MODE_ERI>(P); }
__global__ void __launch_bounds__(128, 2) rys_eri_kernel_ip1(CGLaunch P) { rys_eri_body<CG_MODE_IP1>(P); }
__global__ void __launch_bounds__(128, 2) rys_eri_kernel_ip2(CGLaunch P) { rys_eri_body<CG_MODE_IP2>(P); }
__global__ void __launch_bounds__(128, 2) rys_eri_kernel_ipip1(CGLaunch P) { rys_eri_body<CG_MODE_IPIP1>(P); }
__global__ void __launch_bounds__(128, 2) rys_eri_kernel_prim(CGLaunch P) { rys_eri_body<CG_MODE_ERIP>(P); }

static void *eri_kernel_of(int mode)
{
    return mode == CG_MODE_ERI ? (void *)rys_eri_kernel_e0f0
         : mode == CG_MODE_IP1 ? (void *)rys_eri_kernel_ip1
         : mode == CG_MODE_IP2 ? (void *)rys_eri_kernel_ip2
         : mode == CG_MODE_IPIP1 ? (void *)rys_eri_kernel_ipip1 : (void *)rys_eri_kernel_prim;
}

/* ------------------------------------------------------------------ output kernel */
__global__ void __launch_bounds__(128)
cg_output_kernel(const CGOutTask *__restrict__ ot, const int *__restrict__ idx, int nout,
                 double *gctr, const int *nonempty, double *scratch, int64_t scratch_per_warp,
                 int64_t nf_max, const CGEriClass *__restrict__ eclass,
                 const int *__restrict__ eperm, const int *__restrict__ hprog, double *out,
                 int ncomp, int64_t comp_stride)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double *s1 = scratch + (size_t)gw * scratch_per_warp;
    for (int k = gw; k < nout; k += nw) {
        const int q = idx ? idx[k] : k;
        cg_out_quartet(ot[q], nonempty[q] != 0, false, gctr, eclass, eperm, hprog, out, ncomp,
                       comp_stride, s1, nf_max, scratch_per_warp, lane);
    }
}

/* ------------------------------------------------------------------ host-side launchers */
extern "C" int cg_kernels_init(const int *c2s_nnz, const int *c2s_idx, const double *c2s_val,
                               double **rys_coef_dev)
{
    int rc = cg_tu_tables_init(c2s_nnz, c2s_idx, c2s_val);
    if (rc) return rc;
    rc = cg_grad_tu_init(c2s_nnz, c2s_idx, c2s_val);
    if (rc) return rc;
    cudaError_t e;
    /* the root table lives in the module image; no device allocation at initialisation */
    if ((e = cudaMemcpyToSymbol(g_rys_coef, rys_coef_host, sizeof(double) * RYS_NCOEF)) != cudaSuccess) return (int)e;
    double *d = nullptr;
    if ((e = cudaGetSymbolAddress((void **)&d, g_rys_coef)) != cudaSuccess) return (int)e;
    *rys_coef_dev = d;
    for (int mode : {CG_MODE_ERI, CG_MODE_IP1, CG_MODE_IP2, CG_MODE_IPIP1, CG_MODE_ERIP}) {
        e = cudaFuncSetAttribute(eri_kernel_of(mode), cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * 8 * CG_WS_MAX);
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

extern "C" int cg_blocks_per_sm(int mode, int ws_doubles)
{
    int nb = 0;
    size_t smem = (size_t)4 * ws_doubles * sizeof(double);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, eri_kernel_of(mode), 128, smem) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

extern "C" int cg_rys_nmax(void) { return RYS_NMAX; }
extern "C" int cg_rys_deg(void) { return RYS_DEG; }

extern "C" void cg_layout(int li, int lj, int lk, int ll, int mode, int ws_doubles, CGLayout *L)
{
    cg_class_layout(li, lj, lk, ll, mode, ws_doubles, L);
}

extern "C" int cg_launch_eri(const CGLaunch *P, int mode, int nblocks, cudaStream_t stream)
{
    size_t smem = (size_t)4 * P->ws_doubles * sizeof(double);
    if (mode == CG_MODE_ERI)
        rys_eri_kernel_e0f0<<<nblocks, 128, smem, stream>>>(*P);
    else if (mode == CG_MODE_IP1)
        rys_eri_kernel_ip1<<<nblocks, 128, smem, stream>>>(*P);
    else if (mode == CG_MODE_IP2)
        rys_eri_kernel_ip2<<<nblocks, 128, smem, stream>>>(*P);
    else if (mode == CG_MODE_IPIP1)
        rys_eri_kernel_ipip1<<<nblocks, 128, smem, stream>>>(*P);
    else
        rys_eri_kernel_prim<<<nblocks, 128, smem, stream>>>(*P);
    return (int)cudaGetLastError();
}

extern "C" int cg_launch_output(const CGOutTask *ot, const int *idx, int nout, double *gctr, const int *nonempty,
                                double *scratch, int64_t scratch_per_warp, int64_t nf_max,
                                const CGEriClass *eclass, const int *eperm, const int *hprog,
                                int nblocks, double *out, int ncomp, int64_t comp_stride,
                                cudaStream_t stream)
{
    cg_output_kernel<<<nblocks, 128, 0, stream>>>(ot, idx, nout, gctr, nonempty, scratch,
                                                  scratch_per_warp, nf_max, eclass, eperm, hprog,
                                                  out, ncomp, comp_stride);
    return (int)cudaGetLastError();
}

extern "C" int cg_launch_roots(const double *xs, int count, int n, const double *coef, double *s,
                               double *w, cudaStream_t stream)
{
    if (n < 1 || n > RYS_NMAX) return -1;
    rys_roots_kernel<<<(count + 127) / 128, 128, 0, stream>>>(xs, count, n, coef, s, w);
    return (int)cudaGetLastError();
}
