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

        const int nterm = tk.npq * n;
        for (int t0 = 0; t0 < nterm; t0 += T) {
            const int Tb = min(T, nterm - t0);
            if (lane < Tb) {
                int g = t0 + lane;
                int p = g / n, r = g - p * n;
                int q = __ldg(pql + p);
                int kl = q / nij, ij = q - kl * nij;
                const CGPrimPair A = ppij[ij];
                const CGPrimPair B = ppkl[kl];
                double *rec = term + lane * CG_TERMW_GRAD;
                cg_term(A, B, pij, pkl, n, r, common, P.rys_coef, rec, P.omega2);
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
    return (int)e;
}

extern "C" int cg_grad_blocks_per_sm(int mode, int ws_doubles)
{
    int nb = 0;
    size_t smem = (size_t)4 * ws_doubles * sizeof(double);
    void *fn = mode == CG_MODE_GRAD ? (void *)rys_grad_kernel<CG_MODE_GRAD> : (void *)rys_grad_kernel<CG_MODE_GRADA>;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, smem) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

extern "C" int cg_launch_grad(const CGGradLaunch *P, int mode, int nblocks, cudaStream_t stream)
{
    size_t smem = (size_t)4 * P->ws_doubles * sizeof(double);
    if (mode == CG_MODE_GRAD)
        rys_grad_kernel<CG_MODE_GRAD><<<nblocks, 128, smem, stream>>>(*P);
    else
        rys_grad_kernel<CG_MODE_GRADA><<<nblocks, 128, smem, stream>>>(*P);
    return (int)cudaGetLastError();
}
