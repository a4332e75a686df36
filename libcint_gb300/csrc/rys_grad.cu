/*
 * Adjoint (backward) kernel of the Coulomb-like energy L = 1/2 sum D_ij (ij|kl) D_kl.
 *
 * For every unique shell quartet (weight w_q = 2^[I!=J] 2^[K!=L] 2^[IJ!=KL]) the cotangent of the
 * Cartesian block is W[i,j,k,l] = (w_q / 2) D_ij D_kl (the spherical density pulled back through
 * the cart -> sph matrices on the host).  The kernel recomputes the Rys roots and g arrays of each
 * surviving primitive quartet with the angular momenta raised by one on centres I, J, K (and by two
 * on all four for exponent derivatives) -- libcint's ip1 construction (src/autocode/grad2.c:19-68,
 * CINTnabla1i_2e src/g2e.c:4550-4591) and x1 construction (r^2 insertion, src/g2e.c:4755-4893) --
 * and never stores a derivative integral.  The contraction is organised per axis:
 *
 *   H_a[u] = sum_{components c with a-axis powers u} W[c] g_b[b(c)] g_c[c(c)]
 *   dL/dA_a += H_a[u] (2 a_I g_a[u + e_I] - u_I g_a[u - e_I])       (A = centre of I; J, K alike)
 *   dL/da_s -= H_a[u] g_a[u + 2 e_s]                                 (primitive exponent of shell s)
 *
 * so each Cartesian component costs 3 FP64 operations per axis and root, independent of how many
 * derivatives are taken.  The fourth centre follows from translational invariance.
 * Work items are (term, chunk): a chunk is <= 16 components sharing one a-axis tuple, listed in
 * host-built per-class tables (CGGradChunk/CGGradEnt: g offsets of the partner axes and the
 * component index) sorted longest first, so a round of lanes runs chunks of similar length.  Every
 * quantity downstream of H is linear in H, so chunks of one tuple contribute independently.
 * W (the cotangent per component) is formed once per task, in shared memory up to (dd|dd).
 */
#include "rys_device.cuh"

template <int MODE>
__global__ void __launch_bounds__(128, 2)   /* 2 CTAs/SM (shared memory); no register cap below 255 */
rys_grad_kernel(CGGradLaunch P)
{
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    double *ws = smem + (size_t)warp * P.ws_doubles;
    double *term = ws;                                  /* T * CG_TERMW_GRAD */
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;

    for (;;) {
        int tid = 0;
        if (lane == 0) tid = atomicAdd(P.counter, 1);
        tid = __shfl_sync(FULL, tid, 0);
        if (tid >= P.ntasks) break;
        const CGTask tk = P.tasks[tid];
        const CGPair pij = P.pairs[tk.pij];
        const CGPair pkl = P.pairs[tk.pkl];
        const int li = pij.la, lj = pij.lb, lk = pkl.la, ll = pkl.lb;
        CGLayout L;
        cg_class_layout(li, lj, lk, ll, MODE, P.ws_doubles, &L);
        if (L.T < 1) {
            if (lane == 0) atomicOr(P.status, 1);
            continue;
        }
        const int T = L.T, n = L.nroots, G = L.gax;   /* axis stride of a term's g arrays */
        double *Dij = ws + L.off_dij, *Dkl = ws + L.off_dkl, *aacc = ws + L.off_aacc;
        const int nfi = ncart(li), nfj = ncart(lj), nfk = ncart(lk), nfl = ncart(ll);
        const int nao = P.nao;
        const CGPrimPair *__restrict__ ppij = P.prims + pij.prim_off;
        const CGPrimPair *__restrict__ ppkl = P.prims + pkl.prim_off;
        const int *__restrict__ pql = P.pqlist + tk.pq_off;
        const int nij = pij.npa * pij.npb;
        const double common = P.common_base * common_fac_sp(li) * common_fac_sp(lj)
                            * common_fac_sp(lk) * common_fac_sp(ll);
        const double wq = 0.5 * ((tk.sym & 1) ? 2.0 : 1.0) * ((tk.sym & 2) ? 2.0 : 1.0)
                        * ((tk.sym & 4) ? 2.0 : 1.0);
        for (int e = lane; e < nfi * nfj; e += 32) {
            int i = e / nfj, j = e - i * nfj;
            Dij[e] = wq * __ldg(P.dm + (size_t)(pij.ao_a + i) * nao + pij.ao_b + j);
        }
        for (int e = lane; e < nfk * nfl; e += 32) {
            int k = e / nfl, l = e - k * nfl;
            Dkl[e] = __ldg(P.dm + (size_t)(pkl.ao_a + k) * nao + pkl.ao_b + l);
        }
        if (MODE == CG_MODE_GRADA)
            for (int e = lane; e < 4 * CG_GRAD_MAXPRIM; e += 32) aacc[e] = 0.0;
        __syncwarp();
        /* cotangent of every Cartesian component, c = ((i nfj + j) nfk + k) nfl + l */
        double *W = L.nf <= CG_W_SMEM ? ws + L.off_w : P.wglobal + (size_t)gw * P.wstride;
        for (int c = lane; c < L.nf; c += 32) {
            int l = c % nfl, r = c / nfl;
            int k = r % nfk; r /= nfk;
            W[c] = Dij[r] * Dkl[k * nfl + l];
        }
        const CGGradClass cl = P.gclass[tk.cls];
        const CGGradChunk *__restrict__ chunks = P.gchunk + cl.chunk_off;
        const CGGradEnt *__restrict__ ents = P.gent;
        double *greg = ws + L.off_g;
        __syncwarp();
        double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
        const int sI = L.dJ * L.dK * L.dL, sJ = L.dK * L.dL, sK = L.dL;

        const int nt = P.omega2 < 0.0 ? 2 * n : n;   /* terms per primitive quartet */
        const int nterm = tk.npq * nt;
        for (int t0 = 0; t0 < nterm; t0 += T) {
            const int Tb = min(T, nterm - t0);
            if (lane < Tb) {
                int g = t0 + lane;
                int p = g / nt, r = g - p * nt;
                int q = __ldg(pql + p);
                int kl = q / nij, ij = q - kl * nij;
                const CGPrimPair A = ppij[ij];
                const CGPrimPair B = ppkl[kl];
                double *rec = term + lane * CG_TERMW_GRAD;
                cg_term(A, B, pij, pkl, n, r, common, P.rys_coef, rec, P.omega2, P.expcut);
                rec[10] = 2.0 * A.aA;
                rec[11] = 2.0 * (A.a - A.aA);
                rec[12] = 2.0 * B.aA;
                rec[13] = 2.0 * (B.a - B.aA);
                if (MODE == CG_MODE_GRADA) {
                    int *ri = reinterpret_cast<int *>(rec + 14);
                    ri[0] = ij % pij.npa;
                    ri[1] = ij / pij.npa;
                    ri[2] = kl % pkl.npa;
                    ri[3] = kl / pkl.npa;
                }
            }
            __syncwarp();
            for (int item = lane; item < 3 * Tb; item += 32) {
                int t = item / 3, ax = item - 3 * t;
                const double *rec = term + t * CG_TERMW_GRAD;
                double g00 = (ax == 2) ? rec[9] : 1.0;
                g_axis(L, rec[0], rec[1], rec[2], rec[3 + ax], rec[6 + ax], g00, pij.AB[ax],
                       pkl.AB[ax], ws + L.off_scr + lane * L.scr, greg + (size_t)t * L.gstride + ax * G);
            }
            __syncwarp();
            /* items: (term, chunk); chunks are longest first so a round of lanes runs chunks of
             * similar length */
            const int items = Tb * cl.nchunk;
            for (int base = 0; base < items; base += 32) {
                const int it = base + lane;
                const bool act = it < items;
                /* coordinates only: chunk-major order (a round of lanes shares one chunk and its
                 * length across terms); exponents: term-major, so a round usually holds one term
                 * and its four primitive sums reduce across the warp */
                int t, k;
                if (MODE == CG_MODE_GRAD) { k = it / Tb; t = it - k * Tb; }
                else { t = it / cl.nchunk; k = it - t * cl.nchunk; }
                if (!act) { t = (MODE == CG_MODE_GRAD) ? 0 : Tb - 1; k = 0; }
                double al0 = 0.0, al1 = 0.0, al2 = 0.0, al3 = 0.0;
                if (act) {
                const CGGradChunk &ch = chunks[k];
                const int a = ch.axis_u & 3;
                const int b = a == 2 ? 0 : a + 1, c = 3 - a - b;
                const double *gt = greg + (size_t)t * L.gstride;
                const double *ga = gt + a * G;
                const double *gb = gt + b * G;
                const double *gc = gt + c * G;
                double H = 0.0;
                const int2 *ep = reinterpret_cast<const int2 *>(ents) + ch.ent;
                const int len = ch.len;
                for (int e = 0; e < len; e++) {
                    const int2 en = __ldg(ep + e);
                    H = fma(W[en.y] * gb[en.x & 0xffff], gc[en.x >> 16], H);
                }
                const double *rec = term + t * CG_TERMW_GRAD;
                const int ou = ch.ou;
                double dA = fma(-ch.p[0], ga[ch.om[0]], rec[10] * ga[ou + sI]);
                double dB = fma(-ch.p[1], ga[ch.om[1]], rec[11] * ga[ou + sJ]);
                double dC = fma(-ch.p[2], ga[ch.om[2]], rec[12] * ga[ou + sK]);
                /* the axis is a runtime value: select the accumulators (registers, not a local
                 * array indexed at run time) */
                double xa = a == 0 ? gA[0] : (a == 1 ? gA[1] : gA[2]);
                double xb = a == 0 ? gB[0] : (a == 1 ? gB[1] : gB[2]);
                double xc = a == 0 ? gC[0] : (a == 1 ? gC[1] : gC[2]);
                xa = fma(H, dA, xa);
                xb = fma(H, dB, xb);
                xc = fma(H, dC, xc);
                if (a == 0) { gA[0] = xa; gB[0] = xb; gC[0] = xc; }
                else if (a == 1) { gA[1] = xa; gB[1] = xb; gC[1] = xc; }
                else { gA[2] = xa; gB[2] = xb; gC[2] = xc; }
                if (MODE == CG_MODE_GRADA) {
                    al0 = -H * ga[ou + 2 * sI];
                    al1 = -H * ga[ou + 2 * sJ];
                    al2 = -H * ga[ou + 2 * sK];
                    al3 = -H * ga[ou + 2];
                }
                }
                if (MODE == CG_MODE_GRADA) {
                    /* exponent derivatives belong to the term's four primitives: one warp sum when
                     * the round holds a single term, shared-memory atomics otherwise */
                    const int t_first = __shfl_sync(FULL, t, 0);
                    if (__all_sync(FULL, t == t_first)) {
                        for (int o = 16; o > 0; o >>= 1) {
                            al0 += __shfl_xor_sync(FULL, al0, o);
                            al1 += __shfl_xor_sync(FULL, al1, o);
                            al2 += __shfl_xor_sync(FULL, al2, o);
                            al3 += __shfl_xor_sync(FULL, al3, o);
                        }
                        if (lane == 0) {
                            const double *rec = term + t_first * CG_TERMW_GRAD;
                            const int *ri = reinterpret_cast<const int *>(rec + 14);
                            aacc[0 * CG_GRAD_MAXPRIM + ri[0]] += al0;
                            aacc[1 * CG_GRAD_MAXPRIM + ri[1]] += al1;
                            aacc[2 * CG_GRAD_MAXPRIM + ri[2]] += al2;
                            aacc[3 * CG_GRAD_MAXPRIM + ri[3]] += al3;
                        }
                        __syncwarp();
                    } else if (act) {
                        const double *rec = term + t * CG_TERMW_GRAD;
                        const int *ri = reinterpret_cast<const int *>(rec + 14);
                        atomicAdd(aacc + 0 * CG_GRAD_MAXPRIM + ri[0], al0);
                        atomicAdd(aacc + 1 * CG_GRAD_MAXPRIM + ri[1], al1);
                        atomicAdd(aacc + 2 * CG_GRAD_MAXPRIM + ri[2], al2);
                        atomicAdd(aacc + 3 * CG_GRAD_MAXPRIM + ri[3], al3);
                    }
                }
            }
            __syncwarp();
        }
        /* warp sums of the nine coordinate derivatives; D by translational invariance */
#pragma unroll
        for (int a = 0; a < 3; a++) {
            double x = gA[a], y = gB[a], z = gC[a];
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(FULL, x, o);
                y += __shfl_xor_sync(FULL, y, o);
                z += __shfl_xor_sync(FULL, z, o);
            }
            if (lane == 0) {
                atomicAdd(P.grad + pij.atom_a * 3 + a, x);
                atomicAdd(P.grad + pij.atom_b * 3 + a, y);
                atomicAdd(P.grad + pkl.atom_a * 3 + a, z);
                atomicAdd(P.grad + pkl.atom_b * 3 + a, -(x + y + z));
            }
        }
        if (MODE == CG_MODE_GRADA) {
            __syncwarp();
            const int np[4] = {pij.npa, pij.npb, pkl.npa, pkl.npb};
            const int gp[4] = {pij.gp_a, pij.gp_b, pkl.gp_a, pkl.gp_b};
            for (int e = lane; e < 4 * CG_GRAD_MAXPRIM; e += 32) {
                int s = e / CG_GRAD_MAXPRIM, p = e - s * CG_GRAD_MAXPRIM;
                if (p < np[s] && aacc[e] != 0.0) atomicAdd(P.galpha + gp[s] + p, aacc[e]);
            }
        }
        __syncwarp();
    }
}

/* ------------------------------------------------------------------------------------------
 * Contraction-first adjoint, CG_MODE_GRADJ (coordinates) and CG_MODE_GRADAJ (and exponents).
 *
 * The energy of one unique quartet is E = sum D_ij D_kl (ij|kl) (w_q folded into D_ij).  The
 * horizontal transfer is linear and depends only on AB = A - B (bra) and CD = C - D (ket):
 * (ij| = sum_e Tb(AB)[ij, e] (e0|, with Tb the binomial expansion of (x - B) = (x - A) + AB on
 * each axis (libcint's CINTg0_2e_lj2d4d relation, src/g2e.c:560-693, applied symbolically).  So
 * E = sum_{e,f} De Df (e0|f0) with the transferred densities De = sum_ij D_ij Tb[ij, e] and
 * Df = sum_kl D_kl Tk[kl, f], formed once per task.  Differentiating every factor that moves:
 *
 * The nabla of libcint (src/g2e.c:4550-4591) acts on one shell's Gaussian: A moves only phi_i,
 * (nabla_A i j| = 2a (i+1x j| - i_x (i-1x j|, and the transfer of (i+1x j| is the transfer of
 * (ij| shifted by 1x, that of i_x (i-1x j| the transfer of the i_x-weighted density shifted back;
 * B moves only phi_j, 2b (i j+1x| = 2b [(i+1x j| + AB_x (ij|] and j_x (i j-1x| is the transfer
 * of the AB-derivative of Tb.  So with per-task densities De, iDe_x = sum_ij i_x D_ij Tb[ij, e]
 * and dDe_x = d De / d AB_x (all sums of positive binomial terms, no cancellation):
 *
 *   dE/dA_x = sum_ef Df [2a De[e-1x] (e0|f0) - iDe_x[e+1x] (e0|f0)]
 *   dE/dB_x = sum_ef Df [2b (De[e-1x] + AB_x De[e]) (e0|f0) - dDe_x[e] (e0|f0)]
 *   dE/dC_x = sum_ef De [2c Df[f-1x] (e0|f0) - iDf_x[f+1x] (e0|f0)]
 *
 * (a, b, c: the term's primitive exponents on I, J, K; D by translational invariance).  Writing
 * the A term instead as the derivative of (e0| plus that of De(AB) gives two large contributions
 * that cancel.  Conditioning: for a primitive pair with product centre P, the transfer's binomial
 * terms exceed the result by ((|PA| + |AB|) / |PB|)^lb = (1 + 2 b / a)^lb, harmless when the base
 * primitive a is the tighter one and ruinous when it is a diffuse partner of a tight b (contracted
 * shells mix both: 8e-8 of a c4 gradient).  So every primitive pair expands about its tighter
 * primitive: the planner groups a quartet's primitive quartets by the two choices (bra, ket) into
 * separate tasks, and a task with bit 3 (4) of sym set sees its bra (ket) pair from the second
 * centre.  Per term the bra quantities need
 * only Phi[e'] = sum_f Df (e'0|f0) for |e'| in [li-1, li+lj+1], contracted axis by axis (sum
 * factorisation: z, then y, then x), and the ket ones Psi[f'] = sum_e De (e0|f'0) likewise:
 *
 *   Om[fx,fy][ez'] = sum_fz Df[f] gz(ez', fz)      Xi[fx][ey',ez'] = sum_fy gy(ey', fy) Om[fx,fy][ez']
 *   Phi[e']        = sum_fx gx(ex', fx) Xi[fx][ey',ez']
 *
 * The derivative weights are linear in Phi, so only S1 = sum Phi, Sa = sum 2a Phi and
 * Sb = sum 2b Phi over the task's terms are kept (per e', by the lane owning e'), and the weights
 * are applied once per task:
 *
 *   dE/dA_x = sum_e' Sa[e'] De[e'-1x] - S1[e'] iDe_x[e'+1x]
 *   dE/dB_x = sum_e' Sb[e'] (De[e'-1x] + AB_x De[e']) - S1[e'] dDe_x[e']
 *
 * (C likewise from Psi).  Exponent derivatives (coefficients fixed): the base shell's exponent a
 * multiplies its Gaussian by -|r-A|^2, so dE/da = -sum_x sum_e De Phi[e+2x]; the partner's b by
 * -|r-B|^2 = -sum_x ((x-A_x)^2 + 2 AB_x (x-A_x) + AB_x^2) (the x1 insertion of libcint,
 * src/g2e.c:4755-4893, in the transferred basis).  These go to the term's own primitives, so they
 * are reduced over the warp per term (Phi to |e'| = li+lj+2, Psi likewise).  No Cartesian
 * component of (ij|kl) is formed: the cost per term grows like l^5 instead of the l^8 of the
 * per-component adjoint above.
 * ------------------------------------------------------------------------------------------ */
__constant__ double c_binom5[5][5] = {{1, 0, 0, 0, 0}, {1, 1, 0, 0, 0}, {1, 2, 1, 0, 0},
                                      {1, 3, 3, 1, 0}, {1, 4, 6, 4, 1}};

__device__ __forceinline__ double ipow_small(double x, int p)
{
    double r = 1.0;
    for (int i = 0; i < p; i++) r *= x;
    return r;
}

/* Transferred density of one pair (shells la at A, lb at B = A - AB), tetrahedron layout over
 * |e| <= la + lb (zero below la): Dout[e] = sum_ij w D_ij Tb[ij, e], the transfers of the
 * i_x-weighted density iDout[ax][e] = sum_ij i_ax w D_ij Tb[ij, e] and, when dDout is given, the
 * derivatives along AB dDout[ax][e].  One lane per e. */
__device__ __forceinline__ void cg_pair_density(const double *__restrict__ dm, int nao, const CGPair &pr,
                                                double w, double *Dout, double *iDout, double *dDout,
                                                int lane)
{
    const int la = pr.la, lb = pr.lb, L = la + lb, t = cg_ntet(L);
    const int nfa = ncart(la), nfb = ncart(lb);
    for (int e = lane; e < t; e += 32) {
        int ex, ey, ez;
        cg_dec3(L, e, ex, ey, ez);
        double v = 0.0, d0 = 0.0, d1 = 0.0, d2 = 0.0, i0 = 0.0, i1 = 0.0, i2 = 0.0;
        if (ex + ey + ez >= la) {
            for (int ci = 0; ci < nfa; ci++) {
                int ix, iy, iz;
                cart_pow(la, ci, ix, iy, iz);
                const int kx = ex - ix, ky = ey - iy, kz = ez - iz;
                if (kx < 0 || ky < 0 || kz < 0) continue;
                for (int cj = 0; cj < nfb; cj++) {
                    int jx, jy, jz;
                    cart_pow(lb, cj, jx, jy, jz);
                    const int px = jx - kx, py = jy - ky, pz = jz - kz;
                    if (px < 0 || py < 0 || pz < 0) continue;
                    const double d = w * __ldg(dm + (size_t)(pr.ao_a + ci) * nao + pr.ao_b + cj);
                    const double c = d * c_binom5[jx][kx] * c_binom5[jy][ky] * c_binom5[jz][kz];
                    const double qx = ipow_small(pr.AB[0], px), qy = ipow_small(pr.AB[1], py);
                    const double qz = ipow_small(pr.AB[2], pz);
                    const double t = c * qx * (qy * qz);
                    v += t;
                    i0 = fma((double)ix, t, i0);
                    i1 = fma((double)iy, t, i1);
                    i2 = fma((double)iz, t, i2);
                    if (dDout) {
                        if (px) d0 = fma(c * (double)px * ipow_small(pr.AB[0], px - 1), qy * qz, d0);
                        if (py) d1 = fma(c * (double)py * ipow_small(pr.AB[1], py - 1), qx * qz, d1);
                        if (pz) d2 = fma(c * (double)pz * ipow_small(pr.AB[2], pz - 1), qx * qy, d2);
                    }
                }
            }
        }
        Dout[e] = v;
        iDout[e] = i0;
        iDout[t + e] = i1;
        iDout[2 * t + e] = i2;
        if (dDout) {
            dDout[e] = d0;
            dDout[t + e] = d1;
            dDout[2 * t + e] = d2;
        }
    }
}

/* One side's coordinate weights applied to its sums (lane-owned entries e', tetrahedron index
 * space Lidx >= L + 1; entries with emin <= |e'| <= L + 1):
 * gP_x += sum Sp[e'] D[e'-1x] - S1[e'] iD_x[e'+1x] for the base centre and, with Sq given,
 * gQ_x += sum Sq[e'] (D[e'-1x] + AB_x D[e']) - S1[e'] dD_x[e'] for the partner. */
__device__ __forceinline__ void cg_side_weights(const double *D, const double *iD, const double *dD, int L,
                                                int Lidx, int emin, const double *AB, const double *S1,
                                                const double *Sp, const double *Sq, double gP[3],
                                                double gQ[3], int lane)
{
    const int t = cg_ntet(L), t1 = cg_ntet(Lidx);
    for (int e = lane; e < t1; e += 32) {
        int x[3];
        cg_dec3(Lidx, e, x[0], x[1], x[2]);
        const int s = x[0] + x[1] + x[2];
        if (s < emin || s > L + 1) continue;
        const int me = s <= L ? cg_idx3(L, x[0], x[1], x[2]) : -1;
        const double d0 = me >= 0 ? D[me] : 0.0;
        const double s1 = S1[e], sp = Sp[e], sq = Sq ? Sq[e] : 0.0;
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            int y[3] = {x[0], x[1], x[2]};
            double ip = 0.0, dmn = 0.0;
            if (s + 1 <= L) { y[ax]++; ip = iD[ax * t + cg_idx3(L, y[0], y[1], y[2])]; y[ax]--; }
            if (x[ax] >= 1) { y[ax]--; dmn = D[cg_idx3(L, y[0], y[1], y[2])]; }
            gP[ax] += fma(sp, dmn, -s1 * ip);
            if (Sq) {
                const double tt = me >= 0 ? dD[ax * t + me] : 0.0;
                gQ[ax] += fma(sq, fma(AB[ax], d0, dmn), -s1 * tt);
            }
        }
    }
}

/* Exponent weights of one side over the tetrahedron index space Lidx = L + 2: the base shell's
 * primitive exponent a enters as -|r-A|^2 on its Gaussian, the partner's b as
 * -|r-B|^2 = -sum_x ((x-A_x)^2 + 2 AB_x (x-A_x) + AB_x^2):
 *   Wp[e'] = -sum_x D[e'-2x],   Wq[e'] = -sum_x (D[e'-2x] + 2 AB_x D[e'-1x] + AB_x^2 D[e']) */
__device__ __forceinline__ void cg_side_exp_weights(const double *D, int L, const double *AB, double *Wp,
                                                    double *Wq, int lane)
{
    const int t2 = cg_ntet(L + 2);
    for (int e = lane; e < t2; e += 32) {
        int x[3];
        cg_dec3(L + 2, e, x[0], x[1], x[2]);
        const int s = x[0] + x[1] + x[2];
        const double d0 = s <= L ? D[cg_idx3(L, x[0], x[1], x[2])] : 0.0;
        double wp = 0.0, wq = 0.0;
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            int y[3] = {x[0], x[1], x[2]};
            double d1 = 0.0, d2 = 0.0;
            if (x[ax] >= 1 && s - 1 <= L) { y[ax] -= 1; d1 = D[cg_idx3(L, y[0], y[1], y[2])]; y[ax] += 1; }
            if (x[ax] >= 2) { y[ax] -= 2; d2 = D[cg_idx3(L, y[0], y[1], y[2])]; }
            wp -= d2;
            wq -= fma(AB[ax], fma(AB[ax], d0, 2.0 * d1), d2);
        }
        Wp[e] = wp;
        Wq[e] = wq;
    }
}

/* Sum over the warp of two values per lane: x to lane 0, y to lane 16 (recursive halving) */
__device__ __forceinline__ double cg_warp_sum2(double x, double y, int lane)
{
    double v = (lane & 16) ? y : x;
    const double w = (lane & 16) ? x : y;
    v += __shfl_xor_sync(FULL, w, 16);
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

/* The same shell pair seen from its second centre: base and partner exchanged (AB -> -AB; the
 * primitive pair records stay those of the original order) */
__device__ __forceinline__ void cg_swap_pair(CGPair &p)
{
    for (int c = 0; c < 3; c++) {
        p.A[c] -= p.AB[c];
        p.AB[c] = -p.AB[c];
    }
    int t;
    t = p.la; p.la = p.lb; p.lb = t;
    t = p.ao_a; p.ao_a = p.ao_b; p.ao_b = t;
    t = p.atom_a; p.atom_a = p.atom_b; p.atom_b = t;
    t = p.gp_a; p.gp_a = p.gp_b; p.gp_b = t;
    t = p.npa; p.npa = p.npb; p.npb = t;
}

template <bool EXP>
__global__ void __launch_bounds__(128, 2)
rys_gradj_kernel(CGGradLaunch P)
{
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    double *ws = smem + (size_t)warp * P.ws_doubles;
    constexpr int LMODE = EXP ? CG_MODE_GRADAJ : CG_MODE_GRADJ;

    for (;;) {
        int tid = 0;
        if (lane == 0) tid = atomicAdd(P.counter, 1);
        tid = __shfl_sync(FULL, tid, 0);
        if (tid >= P.ntasks) break;
        const CGTask tk = P.tasks[tid];
        /* the task's primitive pairs all expand about their tighter primitive: bit 3 (4) set, the
         * bra (ket) pair's second centre */
        CGPair pij = P.pairs[tk.pij];
        CGPair pkl = P.pairs[tk.pkl];
        const int npa0 = pij.npa, npc0 = pkl.npa;
        const bool swb = (tk.sym >> 3) & 1, swk = (tk.sym >> 4) & 1;
        if (swb) cg_swap_pair(pij);
        if (swk) cg_swap_pair(pkl);
        const int li = pij.la, lj = pij.lb, lk = pkl.la, ll = pkl.lb;
        CGLayout L;
        cg_class_layout(li, lj, lk, ll, LMODE, P.ws_doubles, &L);
        if (L.T < 1) {
            if (lane == 0) atomicOr(P.status, 1);
            continue;
        }
        const int T = L.T, n = L.nroots, gax = L.gax, gstride = L.gstride, bstride = L.scr;
        const int Le = li + lj, Lf = lk + ll, nmax = L.nmax, mmax = L.mmax;
        const int na = nmax + 1, nm = mmax + 1;
        const int tE0 = cg_ntet(Le), tF0 = cg_ntet(Lf), tE = cg_ntet(nmax), tF = cg_ntet(mmax);
        /* per task: transferred densities, then the sums over terms of Phi, 2a Phi, 2b Phi (bra,
         * per e') and of Psi, 2c Psi (ket, per f'); the lane e' mod 32 owns entry e'.  With
         * exponents: the four shells' exponent weights and per-primitive sums. */
        double *De = ws, *iDe = De + tE0, *dDe = iDe + 3 * tE0, *Df = dDe + 3 * tE0, *iDf = Df + tF0;
        double *S1 = iDf + 3 * tF0, *Sa = S1 + tE, *Sb = Sa + tE, *S1k = Sb + tE, *Sc = S1k + tF;
        double *WI = Sc + tF, *WJ = WI + tE, *WK = WJ + tE, *WL = WK + tF;
        double *aacc = WL + tF;
        double *term = ws + L.off_w;
        double *greg = ws + L.off_g;
        double *buf = ws + L.off_scr;
        const int bred = bstride - 64;          /* exponent partials: the last 64 of a term's buffer */
        const CGPrimPair *__restrict__ ppij = P.prims + pij.prim_off;
        const CGPrimPair *__restrict__ ppkl = P.prims + pkl.prim_off;
        const int *__restrict__ pql = P.pqlist + tk.pq_off;
        const int nij = pij.npa * pij.npb;
        const double common = P.common_base * common_fac_sp(li) * common_fac_sp(lj)
                            * common_fac_sp(lk) * common_fac_sp(ll);
        const double wq = 0.5 * ((tk.sym & 1) ? 2.0 : 1.0) * ((tk.sym & 2) ? 2.0 : 1.0)
                        * ((tk.sym & 4) ? 2.0 : 1.0);
        cg_pair_density(P.dm, P.nao, pij, wq, De, iDe, dDe, lane);
        cg_pair_density(P.dm, P.nao, pkl, 1.0, Df, iDf, nullptr, lane);
        for (int e = lane; e < 3 * tE + 2 * tF; e += 32) S1[e] = 0.0;
        if (EXP)
            for (int e = lane; e < 4 * CG_GRAD_MAXPRIM; e += 32) aacc[e] = 0.0;
        __syncwarp();
        if (EXP) {
            cg_side_exp_weights(De, Le, pij.AB, WI, WJ, lane);
            cg_side_exp_weights(Df, Lf, pkl.AB, WK, WL, lane);
            __syncwarp();
        }

        const int nOm = cg_np2(Lf) * na, q2 = cg_np2(nmax);
        const int nOk = cg_np2(Le) * nm, q2k = cg_np2(mmax);
        const int emin = li > 0 ? li - 1 : 0, fmin = lk > 0 ? lk - 1 : 0;
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
                double *rec = term + lane * L.termw;
                cg_term(A, B, pij, pkl, n, r, common, P.rys_coef, rec, P.omega2, P.expcut);
                const double aa = A.aA, ab = A.a - A.aA, ac = B.aA, ad = B.a - B.aA;
                rec[10] = 2.0 * (swb ? ab : aa);   /* the base exponents: 2a, 2b of the bra, 2c */
                rec[11] = 2.0 * (swb ? aa : ab);
                rec[12] = 2.0 * (swk ? ad : ac);
                double mb = 0.0;
                for (int m = 0; m <= mmax; m++) { rec[13 + m] = mb; mb += rec[2]; }
                if (EXP) {
                    /* primitive indices in the (possibly exchanged) base and partner shells */
                    int *ri = reinterpret_cast<int *>(rec + 13 + nm);
                    const int ip = ij % npa0, jp = ij / npa0, kp = kl % npc0, lp = kl / npc0;
                    ri[0] = swb ? jp : ip;
                    ri[1] = swb ? ip : jp;
                    ri[2] = swk ? lp : kp;
                    ri[3] = swk ? kp : lp;
                }
            }
            if (EXP)
                for (int e = lane; e < 64 * Tb; e += 32) buf[(size_t)(e >> 6) * bstride + bred + (e & 63)] = 0.0;
            __syncwarp();
            /* ---- stage 2: VRR, one lane per (term, axis) */
            for (int item = lane; item < 3 * Tb; item += 32) {
                int t = item / 3, ax = item - 3 * t;
                const double *rec = term + t * L.termw;
                vrr_axis(nmax, mmax, rec[0], rec[1], rec + 13, rec[3 + ax], rec[6 + ax],
                         ax == 2 ? rec[9] : 1.0, greg + (size_t)t * gstride + ax * gax);
            }
            __syncwarp();
            /* ---- bra side: Om (z), Xi (y), then Phi (x) into the lane-owned sums */
            for (int it = lane; it < Tb * nOm; it += 32) {
                const int t = it % Tb, r = it / Tb;
                const int ez = r % na, p = r / na;
                int fx, fy;
                cg_dec2(Lf, p, fx, fy);
                const double *gz = greg + (size_t)t * gstride + 2 * gax;
                const double *df = Df + cg_idx3(Lf, fx, fy, 0);
                const int zlo = max(0, lk - fx - fy), zhi = Lf - fx - fy;
                double s = 0.0;
                for (int fz = zlo; fz <= zhi; fz++) s = fma(df[fz], gz[ez + na * fz], s);
                buf[(size_t)t * bstride + p * na + ez] = s;
            }
            __syncwarp();
            for (int it = lane; it < Tb * (Lf + 1) * q2; it += 32) {
                const int t = it % Tb, r = it / Tb;
                const int q = r % q2, fx = r / q2;
                int ey, ez;
                cg_dec2(nmax, q, ey, ez);
                const double *gy = greg + (size_t)t * gstride + gax;
                const double *om = buf + (size_t)t * bstride;
                double s = 0.0;
                for (int fy = 0; fy <= Lf - fx; fy++)
                    s = fma(gy[ey + na * fy], om[cg_idx2(Lf, fx, fy) * na + ez], s);
                buf[(size_t)t * bstride + nOm + fx * q2 + q] = s;
            }
            __syncwarp();
            for (int e = lane; e < tE; e += 32) {
                int x0, x1, x2;
                cg_dec3(nmax, e, x0, x1, x2);
                const int es = x0 + x1 + x2;
                if (es < emin) continue;
                const bool crd = es <= Le + 1, xp = EXP && es >= li;
                const int ixi = nOm + cg_idx2(nmax, x1, x2);
                double s1 = S1[e], sa = Sa[e], sb = Sb[e];
                const double wi = xp ? WI[e] : 0.0, wj = xp ? WJ[e] : 0.0;
                for (int t = 0; t < Tb; t++) {
                    const double *gx = greg + (size_t)t * gstride + x0;
                    const double *xi = buf + (size_t)t * bstride + ixi;
                    double phi = 0.0;
                    for (int fx = 0; fx <= Lf; fx++) phi = fma(gx[na * fx], xi[fx * q2], phi);
                    const double *rec = term + t * L.termw;
                    if (crd) {
                        s1 += phi;
                        sa = fma(rec[10], phi, sa);
                        sb = fma(rec[11], phi, sb);
                    }
                    if (xp) {
                        double *red = buf + (size_t)t * bstride + bred + lane;
                        red[0] = fma(phi, wi, red[0]);
                        red[32] = fma(phi, wj, red[32]);
                    }
                }
                S1[e] = s1;
                Sa[e] = sa;
                Sb[e] = sb;
            }
            __syncwarp();
            if (EXP) {
                /* the bra shells' exponent sums of each term, to its two primitives */
                for (int t = 0; t < Tb; t++) {
                    const double *red = buf + (size_t)t * bstride + bred + lane;
                    const double v = cg_warp_sum2(red[0], red[32], lane);
                    const int *ri = reinterpret_cast<const int *>(term + t * L.termw + 13 + nm);
                    if (lane == 0) aacc[ri[0]] += v;
                    if (lane == 16) aacc[CG_GRAD_MAXPRIM + ri[1]] += v;
                }
                for (int e = lane; e < 64 * Tb; e += 32) buf[(size_t)(e >> 6) * bstride + bred + (e & 63)] = 0.0;
                __syncwarp();
            }
            /* ---- ket side: the same with the pairs' roles exchanged, sums of Psi and 2c Psi */
            for (int it = lane; it < Tb * nOk; it += 32) {
                const int t = it % Tb, r = it / Tb;
                const int fz = r % nm, p = r / nm;
                int ex, ey;
                cg_dec2(Le, p, ex, ey);
                const double *gz = greg + (size_t)t * gstride + 2 * gax;
                const double *de = De + cg_idx3(Le, ex, ey, 0);
                const int zlo = max(0, li - ex - ey), zhi = Le - ex - ey;
                double s = 0.0;
                for (int ez = zlo; ez <= zhi; ez++) s = fma(de[ez], gz[ez + na * fz], s);
                buf[(size_t)t * bstride + p * nm + fz] = s;
            }
            __syncwarp();
            for (int it = lane; it < Tb * (Le + 1) * q2k; it += 32) {
                const int t = it % Tb, r = it / Tb;
                const int q = r % q2k, ex = r / q2k;
                int fy, fz;
                cg_dec2(mmax, q, fy, fz);
                const double *gy = greg + (size_t)t * gstride + gax;
                const double *om = buf + (size_t)t * bstride;
                double s = 0.0;
                for (int ey = 0; ey <= Le - ex; ey++)
                    s = fma(gy[ey + na * fy], om[cg_idx2(Le, ex, ey) * nm + fz], s);
                buf[(size_t)t * bstride + nOk + ex * q2k + q] = s;
            }
            __syncwarp();
            for (int f = lane; f < tF; f += 32) {
                int y0, y1, y2;
                cg_dec3(mmax, f, y0, y1, y2);
                const int fs = y0 + y1 + y2;
                if (fs < fmin) continue;
                const bool crd = fs <= Lf + 1, xp = EXP && fs >= lk;
                const int ixi = nOk + cg_idx2(mmax, y1, y2);
                double s1 = S1k[f], sc = Sc[f];
                const double wk = xp ? WK[f] : 0.0, wl = xp ? WL[f] : 0.0;
                for (int t = 0; t < Tb; t++) {
                    const double *gx = greg + (size_t)t * gstride + na * y0;
                    const double *xi = buf + (size_t)t * bstride + ixi;
                    double psi = 0.0;
                    for (int ex = 0; ex <= Le; ex++) psi = fma(gx[ex], xi[ex * q2k], psi);
                    if (crd) {
                        s1 += psi;
                        sc = fma(term[t * L.termw + 12], psi, sc);
                    }
                    if (xp) {
                        double *red = buf + (size_t)t * bstride + bred + lane;
                        red[0] = fma(psi, wk, red[0]);
                        red[32] = fma(psi, wl, red[32]);
                    }
                }
                S1k[f] = s1;
                Sc[f] = sc;
            }
            __syncwarp();
            if (EXP) {
                for (int t = 0; t < Tb; t++) {
                    const double *red = buf + (size_t)t * bstride + bred + lane;
                    const double v = cg_warp_sum2(red[0], red[32], lane);
                    const int *ri = reinterpret_cast<const int *>(term + t * L.termw + 13 + nm);
                    if (lane == 0) aacc[2 * CG_GRAD_MAXPRIM + ri[2]] += v;
                    if (lane == 16) aacc[3 * CG_GRAD_MAXPRIM + ri[3]] += v;
                }
                __syncwarp();
            }
        }
        /* the coordinate weights, once per task */
        double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
        cg_side_weights(De, iDe, dDe, Le, nmax, emin, pij.AB, S1, Sa, Sb, gA, gB, lane);
        cg_side_weights(Df, iDf, nullptr, Lf, mmax, fmin, pkl.AB, S1k, Sc, nullptr, gC, gC, lane);
        /* warp sums of the nine coordinate derivatives; D by translational invariance */
#pragma unroll
        for (int a = 0; a < 3; a++) {
            double x = gA[a], y = gB[a], z = gC[a];
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(FULL, x, o);
                y += __shfl_xor_sync(FULL, y, o);
                z += __shfl_xor_sync(FULL, z, o);
            }
            if (lane == 0) {
                atomicAdd(P.grad + pij.atom_a * 3 + a, x);
                atomicAdd(P.grad + pij.atom_b * 3 + a, y);
                atomicAdd(P.grad + pkl.atom_a * 3 + a, z);
                atomicAdd(P.grad + pkl.atom_b * 3 + a, -(x + y + z));
            }
        }
        if (EXP) {
            __syncwarp();
            const int np[4] = {pij.npa, pij.npb, pkl.npa, pkl.npb};
            const int gp[4] = {pij.gp_a, pij.gp_b, pkl.gp_a, pkl.gp_b};
            for (int e = lane; e < 4 * CG_GRAD_MAXPRIM; e += 32) {
                int s = e / CG_GRAD_MAXPRIM, p = e - s * CG_GRAD_MAXPRIM;
                if (p < np[s] && aacc[e] != 0.0) atomicAdd(P.galpha + gp[s] + p, aacc[e]);
            }
        }
        __syncwarp();
    }
}

extern "C" int cg_grad_tu_init(const int *c2s_nnz, const int *c2s_idx, const double *c2s_val)
{
    int rc = cg_tu_tables_init(c2s_nnz, c2s_idx, c2s_val);
    if (rc) return rc;
    cudaError_t e;
    e = cudaFuncSetAttribute((void *)rys_grad_kernel<CG_MODE_GRAD>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * 8 * CG_WS_MAX);
    if (e != cudaSuccess) return (int)e;
    e = cudaFuncSetAttribute((void *)rys_grad_kernel<CG_MODE_GRADA>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * 8 * CG_WS_MAX);
    if (e != cudaSuccess) return (int)e;
    e = cudaFuncSetAttribute((void *)rys_gradj_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             4 * 8 * CG_WS_MAX);
    if (e != cudaSuccess) return (int)e;
    e = cudaFuncSetAttribute((void *)rys_gradj_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             4 * 8 * CG_WS_MAX);
    return (int)e;
}

extern "C" int cg_grad_blocks_per_sm(int mode, int ws_doubles)
{
    int nb = 0;
    size_t smem = (size_t)4 * ws_doubles * sizeof(double);
    void *fn = mode == CG_MODE_GRAD ? (void *)rys_grad_kernel<CG_MODE_GRAD>
             : mode == CG_MODE_GRADJ ? (void *)rys_gradj_kernel<false>
             : mode == CG_MODE_GRADAJ ? (void *)rys_gradj_kernel<true> : (void *)rys_grad_kernel<CG_MODE_GRADA>;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, smem) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

extern "C" int cg_launch_grad(const CGGradLaunch *P, int mode, int nblocks, cudaStream_t stream)
{
    size_t smem = (size_t)4 * P->ws_doubles * sizeof(double);
    if (mode == CG_MODE_GRADJ)
        rys_gradj_kernel<false><<<nblocks, 128, smem, stream>>>(*P);
    else if (mode == CG_MODE_GRADAJ)
        rys_gradj_kernel<true><<<nblocks, 128, smem, stream>>>(*P);
    else if (mode == CG_MODE_GRAD)
        rys_grad_kernel<CG_MODE_GRAD><<<nblocks, 128, smem, stream>>>(*P);
    else
        rys_grad_kernel<CG_MODE_GRADA><<<nblocks, 128, smem, stream>>>(*P);
    return (int)cudaGetLastError();
}
