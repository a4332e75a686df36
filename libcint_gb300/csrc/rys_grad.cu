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
 * Work items are (term, axis, a-axis tuple, chunk of at most K partner tuples); every quantity
 * downstream of H is linear in H, so chunks contribute independently and the lanes stay balanced.
 */
#include "rys_device.cuh"

#define GRAD_CHUNK_TABLE 1024

/* chunk size K for a class: at most GRAD_CHUNK_TABLE (tuple, chunk) entries */
__host__ __device__ inline int grad_chunk(int li, int lj, int lk, int ll, int *nchunks)
{
    int l[4] = {li, lj, lk, ll};
    for (int K = 16;; K *= 2) {
        int tot = 0;
        for (int p0 = 0; p0 <= l[0]; p0++)
            for (int p1 = 0; p1 <= l[1]; p1++)
                for (int p2 = 0; p2 <= l[2]; p2++)
                    for (int p3 = 0; p3 <= l[3]; p3++) {
                        int nv = (l[0] - p0 + 1) * (l[1] - p1 + 1) * (l[2] - p2 + 1) * (l[3] - p3 + 1);
                        tot += (nv + K - 1) / K;
                    }
        if (tot <= GRAD_CHUNK_TABLE || K >= 4096) {
            if (nchunks) *nchunks = tot;
            return K;
        }
    }
}

__device__ __forceinline__ int cart_idx(int l, int lx, int ly)
{
    /* CINTcart_comp order: rows of decreasing lx, inside a row decreasing ly */
    int r = l - lx;
    return r * (r + 1) / 2 + (r - ly);
}

template <int MODE>
__global__ void __launch_bounds__(128)
rys_grad_kernel(CGGradLaunch P)
{
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    double *ws = smem + (size_t)warp * P.ws_doubles;
    double *term = ws;                                  /* CG_TERMW_GRAD * 32 */
    double *Dij = term + CG_TERMW_GRAD * 32;            /* 225 */
    double *Dkl = Dij + 225;                            /* 225 */
    double *aacc = Dkl + 225;                           /* 4 * CG_GRAD_MAXPRIM */
    int *ctab = reinterpret_cast<int *>(aacc + 4 * CG_GRAD_MAXPRIM);   /* GRAD_CHUNK_TABLE ints */
    double *greg = aacc + 4 * CG_GRAD_MAXPRIM + GRAD_CHUNK_TABLE / 2;

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
        const int T = L.T, n = L.nroots, G = L.G;
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
        /* (tuple, chunk) table: tuples u = (p0,p1,p2,p3), p0 fastest */
        int nchunk = 0;
        const int K = grad_chunk(li, lj, lk, ll, &nchunk);
        const int nT = (li + 1) * (lj + 1) * (lk + 1) * (ll + 1);
        {
            int base = 0;
            for (int u0 = 0; u0 < nT; u0 += 32) {
                int u = u0 + lane, cnt = 0, p[4];
                if (u < nT) {
                    int r = u;
                    p[0] = r % (li + 1); r /= (li + 1);
                    p[1] = r % (lj + 1); r /= (lj + 1);
                    p[2] = r % (lk + 1); p[3] = r / (lk + 1);
                    int nv = (li - p[0] + 1) * (lj - p[1] + 1) * (lk - p[2] + 1) * (ll - p[3] + 1);
                    cnt = (nv + K - 1) / K;
                }
                int incl = cnt;
                for (int o = 1; o < 32; o <<= 1) {
                    int v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += v;
                }
                int start = base + incl - cnt;
                for (int q = 0; q < cnt; q++) ctab[start + q] = u | (q << 16);
                base += __shfl_sync(FULL, incl, 31);
            }
        }
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
                cg_term(A, B, pij, pkl, n, r, common, P.rys_coef, rec);
                rec[10] = 2.0 * A.aA;
                rec[11] = 2.0 * (A.a - A.aA);
                rec[12] = 2.0 * B.aA;
                rec[13] = 2.0 * (B.a - B.aA);
                rec[14] = (double)(ij % pij.npa);
                rec[15] = (double)(ij / pij.npa);
                rec[16] = (double)(kl % pkl.npa);
                rec[17] = (double)(kl / pkl.npa);
            }
            __syncwarp();
            for (int item = lane; item < 3 * Tb; item += 32) {
                int t = item / 3, ax = item - 3 * t;
                const double *rec = term + t * CG_TERMW_GRAD;
                double g00 = (ax == 2) ? rec[9] : 1.0;
                g_axis(L, rec[0], rec[1], rec[2], rec[3 + ax], rec[6 + ax], g00, pij.AB[ax],
                       pkl.AB[ax], greg + T * 3 * G + lane * L.scr, greg + (size_t)(t * 3 + ax) * G);
            }
            __syncwarp();
            const int items = Tb * 3 * nchunk;
            for (int it = lane; it < items; it += 32) {
                int t = it / (3 * nchunk);
                int rem = it - t * 3 * nchunk;
                int a = rem / nchunk;
                int e = ctab[rem - a * nchunk];
                int u = e & 0xffff, q = e >> 16;
                int p0, p1, p2, p3;
                {
                    int r = u;
                    p0 = r % (li + 1); r /= (li + 1);
                    p1 = r % (lj + 1); r /= (lj + 1);
                    p2 = r % (lk + 1); p3 = r / (lk + 1);
                }
                const int b = a == 2 ? 0 : a + 1, c = 3 - a - b;
                const double *ga = greg + (size_t)(t * 3 + a) * G;
                const double *gb = greg + (size_t)(t * 3 + b) * G;
                const double *gc = greg + (size_t)(t * 3 + c) * G;
                const int r0 = li - p0 + 1, r1 = lj - p1 + 1, r2 = lk - p2 + 1, r3 = ll - p3 + 1;
                const int nv = r0 * r1 * r2 * r3;
                const int v1 = min(nv, (q + 1) * K);
                double H = 0.0;
                for (int v = q * K; v < v1; v++) {
                    int r = v;
                    int b0 = r % r0; r /= r0;
                    int b1 = r % r1; r /= r1;
                    int b2 = r % r2; int b3 = r / r2;
                    int c0 = li - p0 - b0, c1 = lj - p1 - b1, c2 = lk - p2 - b2, c3 = ll - p3 - b3;
                    int ob = ((b0 * L.dJ + b1) * L.dK + b2) * L.dL + b3;
                    int oc = ((c0 * L.dJ + c1) * L.dK + c2) * L.dL + c3;
                    /* x and y powers per shell for the component index */
                    int xI = a == 0 ? p0 : (b == 0 ? b0 : c0), yI = a == 1 ? p0 : (b == 1 ? b0 : c0);
                    int xJ = a == 0 ? p1 : (b == 0 ? b1 : c1), yJ = a == 1 ? p1 : (b == 1 ? b1 : c1);
                    int xK = a == 0 ? p2 : (b == 0 ? b2 : c2), yK = a == 1 ? p2 : (b == 1 ? b2 : c2);
                    int xL = a == 0 ? p3 : (b == 0 ? b3 : c3), yL = a == 1 ? p3 : (b == 1 ? b3 : c3);
                    double W = Dij[cart_idx(li, xI, yI) * nfj + cart_idx(lj, xJ, yJ)]
                             * Dkl[cart_idx(lk, xK, yK) * nfl + cart_idx(ll, xL, yL)];
                    H = fma(W * gb[ob], gc[oc], H);
                }
                const double *rec = term + t * CG_TERMW_GRAD;
                const int ou = ((p0 * L.dJ + p1) * L.dK + p2) * L.dL + p3;
                double dA = rec[10] * ga[ou + sI];
                if (p0) dA = fma(-(double)p0, ga[ou - sI], dA);
                double dB = rec[11] * ga[ou + sJ];
                if (p1) dB = fma(-(double)p1, ga[ou - sJ], dB);
                double dC = rec[12] * ga[ou + sK];
                if (p2) dC = fma(-(double)p2, ga[ou - sK], dC);
                gA[a] = fma(H, dA, gA[a]);
                gB[a] = fma(H, dB, gB[a]);
                gC[a] = fma(H, dC, gC[a]);
                if (MODE == CG_MODE_GRADA) {
                    atomicAdd(aacc + 0 * CG_GRAD_MAXPRIM + (int)rec[14], -H * ga[ou + 2 * sI]);
                    atomicAdd(aacc + 1 * CG_GRAD_MAXPRIM + (int)rec[15], -H * ga[ou + 2 * sJ]);
                    atomicAdd(aacc + 2 * CG_GRAD_MAXPRIM + (int)rec[16], -H * ga[ou + 2 * sK]);
                    atomicAdd(aacc + 3 * CG_GRAD_MAXPRIM + (int)rec[17], -H * ga[ou + 2]);
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
            __syncwarp();
        }
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
