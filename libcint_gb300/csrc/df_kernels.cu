/*
 * Density-fitted Coulomb contractions over the packed three-index buffer.
 *
 * The buffer is what a CINTGPU_INT3C2E_SPH (or _CART) plan writes for the items "orbital shell
 * pair p = (i, j), i >= j, with every auxiliary shell, auxiliary shells in order" (libcint's
 * int3c2e_sph blocks (di, dj, dP), i fastest, src/cint3c2e.c:693-717, back to back): pair p owns
 * one segment of di dj naux doubles in which element (a, b, Q) sits at a + di (b + dj Q), Q the
 * auxiliary function counted from 0.  Pairs follow one another in the order given.
 *
 *   rho_Q  = sum_p w_p sum_ab T_p[ab, Q] D[oi + a, oj + b]      (w_p = 2 for i != j, else 1)
 *   J[oi + a, oj + b] = J[oj + b, oi + a] = sum_Q T_p[ab, Q] c_Q
 *
 * Both contractions read the buffer once with one FP64 FMA per 8-byte element, which on GB300
 * (2 DFMA per SM per clock: 629 G FMA/s) caps them at ~5.0 TB/s, below HBM: the FP64 pipe is
 * their bound, so every FMA runs with all 32 lanes and nothing else per element is FP64.
 *  - rho: the pairs' weighted densities are gathered once per call into one array (w_p D in the
 *    buffer's AO-pair order); then one warp per task (a range of pairs x 128 auxiliary functions,
 *    four per lane) broadcasts them by shuffles (one shuffle per four FMAs), keeps partial sums
 *    over the range in registers and adds them atomically once per function and task;
 *  - J: one warp per pair, lane per auxiliary function, 32 AO-pair partial sums per lane in
 *    registers, one reduce-scatter per 32 AO pairs; each pair owns its blocks of J (no atomics).
 * A lane reads the di dj consecutive elements of its column; the warp's loads of one ab fall on
 * 32 sectors that the next ab's loads hit again in L1, so DRAM sees each byte once.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "cintgpu_internal.h"

#define DF_FULL 0xffffffffu
#define DF_WARPS 8             /* warps per CTA */
#define DF_MAX_AB 4096         /* di dj per pair */

struct CINTGPUDF {
    int64_t npair = 0;
    int naux = 0, nao = 0, max_ab = 0, range = 1;
    int64_t size = 0;          /* doubles of the packed buffer */
    int64_t *d_seg = nullptr;  /* segment start of each pair */
    int4 *d_desc = nullptr;    /* oi, oj, di, dj */
    int *d_order = nullptr;    /* pairs by decreasing di dj (the J kernel's order) */
    int64_t *d_doff = nullptr; /* start of each pair's block in d_dw */
    double *d_dw = nullptr;    /* w_p D[oi + a, oj + b] per pair, ab order (formed per rho call) */
    int64_t nab_total = 0;
    unsigned long long *d_counter = nullptr;
    int blocks_rho = 1, blocks_j = 1;
};

/* b = ab / di (a = ab - b di) for the small non-negative integers of an AO-pair block, through a
 * float estimate and one correction each way (no integer division subroutine) */
__device__ __forceinline__ int df_div(int ab, int di)
{
    int b = (int)__fdividef(ab + 0.5f, (float)di);
    if (b * di > ab) b--;
    if ((b + 1) * di <= ab) b++;
    return b;
}

/* the weighted density of every pair in the buffer's AO-pair order: dw[doff_p + a + di b] =
 * w_p D[oi + a, oj + b] (one warp per pair, lane per AO pair) */
__global__ void __launch_bounds__(32 * DF_WARPS)
df_density_kernel(const int4 *__restrict__ desc, const int64_t *__restrict__ doff, int64_t npair,
                  const double *__restrict__ dm, int nao, double *__restrict__ dw)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * DF_WARPS;
    for (int64_t p = (int64_t)blockIdx.x * DF_WARPS + (threadIdx.x >> 5); p < npair; p += nw) {
        const int4 d = __ldg(desc + p);
        const int nab = d.z * d.w;
        const double w = d.x != d.y ? 2.0 : 1.0;
        double *o = dw + __ldg(doff + p);
        for (int ab = lane; ab < nab; ab += 32) {
            const int b = df_div(ab, d.z);
            o[ab] = w * __ldg(dm + (int64_t)(d.x + ab - b * d.z) * nao + d.y + b);
        }
    }
}

#define DF_QCOL 4              /* auxiliary functions per lane in a rho task (32 x 4 per task) */

/* CNT AO pairs (from j0 of the chunk) of a lane's DF_QCOL columns (cstride apart) times the
 * broadcast density: the loads are issued together, then one shuffle serves DF_QCOL FMAs */
template <int CNT>
__device__ __forceinline__ void df_rho_chunk(const double *__restrict__ e, int64_t cstride, double dd,
                                             int j0, const bool (&on)[DF_QCOL], double (&acc)[DF_QCOL])
{
    double t[CNT][DF_QCOL];
#pragma unroll
    for (int i = 0; i < CNT; i++)
#pragma unroll
        for (int k = 0; k < DF_QCOL; k++) t[i][k] = on[k] ? __ldg(e + i + k * cstride) : 0.0;
#pragma unroll
    for (int i = 0; i < CNT; i++) {
        const double dj = __shfl_sync(DF_FULL, dd, j0 + i);
#pragma unroll
        for (int k = 0; k < DF_QCOL; k++) acc[k] = fma(t[i][k], dj, acc[k]);
    }
}

__global__ void __launch_bounds__(32 * DF_WARPS, 3)
df_rho_kernel(const double *__restrict__ T, const int64_t *__restrict__ seg,
              const int4 *__restrict__ desc, int64_t npair, int range, int naux,
              const int64_t *__restrict__ doff, const double *__restrict__ dw, double *__restrict__ rho)
{
    /* the host keeps nrange x nblk below 2^30, so task indices are 32-bit */
    const int lane = threadIdx.x & 31;
    const int nblk = (naux + 32 * DF_QCOL - 1) / (32 * DF_QCOL);
    const int nrange = (int)((npair + range - 1) / range);
    const int ntask = nrange * nblk;
    const int nw = gridDim.x * DF_WARPS;
    for (int t = blockIdx.x * DF_WARPS + (threadIdx.x >> 5); t < ntask; t += nw) {
        const int r = t / nblk, qb = t - r * nblk;
        const int Q0 = qb * 32 * DF_QCOL + lane;
        bool on[DF_QCOL];
        double acc[DF_QCOL];
#pragma unroll
        for (int k = 0; k < DF_QCOL; k++) { on[k] = Q0 + 32 * k < naux; acc[k] = 0.0; }
        const int64_t p0 = (int64_t)r * range, p1 = min(npair, p0 + range);
        for (int64_t p = p0; p < p1; p++) {
            const int4 d = __ldg(desc + p);
            const int nab = d.z * d.w;
            const double *tp = T + __ldg(seg + p) + (int64_t)nab * (on[0] ? Q0 : 0);
            const double *dp = dw + __ldg(doff + p);
            const int64_t cstride = (int64_t)nab * 32;
            for (int ab0 = 0; ab0 < nab; ab0 += 32) {
                /* the pair's weighted density, one element per lane, broadcast by shuffles */
                const int ab = ab0 + lane;
                const double dd = ab < nab ? __ldg(dp + ab) : 0.0;
                const int cnt = min(32, nab - ab0);
                const double *e = tp + ab0;
                int j0 = 0;
                for (; j0 + 4 <= cnt; j0 += 4) df_rho_chunk<4>(e + j0, cstride, dd, j0, on, acc);
                switch (cnt - j0) {
                case 1: df_rho_chunk<1>(e + j0, cstride, dd, j0, on, acc); break;
                case 2: df_rho_chunk<2>(e + j0, cstride, dd, j0, on, acc); break;
                case 3: df_rho_chunk<3>(e + j0, cstride, dd, j0, on, acc); break;
                default: break;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < DF_QCOL; k++)
            if (on[k]) atomicAdd(rho + Q0 + 32 * k, acc[k]);
    }
}

/* x[0..31] of every lane -> lane l holds the sum over the warp of x[l] (recursive halving: 31
 * adds and 31 shuffles per lane instead of 5 per element) */
__device__ __forceinline__ double df_reduce_scatter32(double (&x)[32], int lane)
{
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool hi = (lane & h) != 0;
#pragma unroll
        for (int i = 0; i < h; i++) {
            const double keep = hi ? x[i + h] : x[i];
            const double send = hi ? x[i] : x[i + h];
            x[i] = keep + __shfl_xor_sync(DF_FULL, send, h);
        }
    }
    return x[0];
}

/* one 32-AO-pair chunk of pair p's J block: lane per auxiliary function, CNT partial sums per
 * lane in registers (one FMA per buffer element, no predicated-off FMAs), then summed over the
 * warp: lane l ends with AO pair ab0 + l */
template <int CNT>
__device__ __forceinline__ double df_j_chunk(const double *__restrict__ tp, int nab, int ab0, int naux,
                                             const double *__restrict__ c, int lane)
{
    double x[32];
#pragma unroll
    for (int i = 0; i < 32; i++) x[i] = 0.0;
    for (int Q = lane; Q < naux; Q += 32) {
        const double cq = __ldg(c + Q);
        const double *e = tp + (int64_t)nab * Q + ab0;
#pragma unroll
        for (int i = 0; i < CNT; i++) x[i] = fma(__ldg(e + i), cq, x[i]);
    }
    if (CNT <= 6) {
        /* a butterfly per AO pair (5 adds each) is cheaper than the 31 of the reduce-scatter */
        double v = 0.0;
#pragma unroll
        for (int i = 0; i < CNT; i++) {
            double y = x[i];
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) y += __shfl_xor_sync(DF_FULL, y, o);
            if (lane == i) v = y;
        }
        return v;
    }
    return df_reduce_scatter32(x, lane);
}

__global__ void __launch_bounds__(32 * DF_WARPS)
df_j_kernel(const double *__restrict__ T, const int64_t *__restrict__ seg,
            const int4 *__restrict__ desc, const int *__restrict__ order, int64_t npair, int naux,
            const double *__restrict__ c, int nao, double *__restrict__ vj, unsigned long long *counter)
{
    /* pairs are taken largest first (order) from a counter, so no warp ends long after the rest */
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(counter, 1ull);
        k = __shfl_sync(DF_FULL, k, 0);
        if (k >= (unsigned long long)npair) break;
        const int64_t p = __ldg(order + k);
        const int4 d = __ldg(desc + p);
        const int nab = d.z * d.w;
        const double *tp = T + __ldg(seg + p);
        for (int ab0 = 0; ab0 < nab; ab0 += 32) {
            const int cnt = min(32, nab - ab0);
            double v;
            switch (cnt) {
#define DF_CASE(n) case n: v = df_j_chunk<n>(tp, nab, ab0, naux, c, lane); break;
            DF_CASE(1) DF_CASE(2) DF_CASE(3) DF_CASE(4) DF_CASE(5) DF_CASE(6) DF_CASE(7) DF_CASE(8)
            DF_CASE(9) DF_CASE(10) DF_CASE(11) DF_CASE(12) DF_CASE(13) DF_CASE(14) DF_CASE(15)
            DF_CASE(16) DF_CASE(17) DF_CASE(18) DF_CASE(19) DF_CASE(20) DF_CASE(21) DF_CASE(22)
            DF_CASE(23) DF_CASE(24) DF_CASE(25) DF_CASE(26) DF_CASE(27) DF_CASE(28) DF_CASE(29)
            DF_CASE(30) DF_CASE(31)
            default: v = df_j_chunk<32>(tp, nab, ab0, naux, c, lane); break;
#undef DF_CASE
            }
            if (lane < cnt) {
                const int ab = ab0 + lane, b = df_div(ab, d.z), a = ab - b * d.z;
                vj[(int64_t)(d.x + a) * nao + d.y + b] = v;
                if (d.x != d.y) vj[(int64_t)(d.y + b) * nao + d.x + a] = v;
            }
        }
    }
}

static int df_fail(const char *msg)
{
    cg_set_error_msg(msg);
    return CINTGPU_ERR_ARG;
}

extern "C" {

int cintgpu_df_create(CINTGPUDF **out, const int *pairs, int64_t npair, int nao, int naux)
{
    if (!out) return df_fail("df: null handle pointer");
    *out = nullptr;
    if (npair < 0 || (npair > 0 && !pairs) || nao < 1 || naux < 1)
        return df_fail("df: need npair >= 0 (with its descriptors), nao >= 1, naux >= 1");
    std::vector<int64_t> seg((size_t)std::max<int64_t>(npair, 1));
    std::vector<int4> desc((size_t)std::max<int64_t>(npair, 1));
    int64_t pos = 0;
    int max_ab = 1;
    for (int64_t p = 0; p < npair; p++) {
        const int oi = pairs[4 * p], oj = pairs[4 * p + 1], di = pairs[4 * p + 2], dj = pairs[4 * p + 3];
        if (oi < 0 || oj < 0 || di < 1 || dj < 1 || oi + di > nao || oj + dj > nao || di * dj > DF_MAX_AB) {
            char m[160];
            snprintf(m, sizeof m, "df: pair %lld (offsets %d, %d, extents %d, %d) outside %d AOs or above %d "
                                  "AO pairs", (long long)p, oi, oj, di, dj, nao, DF_MAX_AB);
            return df_fail(m);
        }
        seg[p] = pos;
        desc[p] = make_int4(oi, oj, di, dj);
        pos += (int64_t)di * dj * naux;
        max_ab = std::max(max_ab, di * dj);
    }
    int rc = cg_init();
    if (rc) return rc;
    CINTGPUDF *h = new CINTGPUDF();
    h->npair = npair;
    h->naux = naux;
    h->nao = nao;
    h->max_ab = max_ab;
    h->size = pos;
    const int sm = std::max(1, cg_sm_count());
    /* rho tasks: ranges of pairs x blocks of 32 DF_QCOL auxiliary functions; ranges long enough
     * that the atomic adds (nrange x naux) stay well below the buffer's elements, short enough for
     * about 8 tasks per resident warp */
    const int64_t nblk = (naux + 32 * DF_QCOL - 1) / (32 * DF_QCOL);
    const int64_t want = (int64_t)sm * 4 * DF_WARPS * 8;
    int64_t range = std::max<int64_t>(4, std::min<int64_t>(4096, npair * nblk / std::max<int64_t>(want, 1)));
    while (((npair + range - 1) / range) * nblk >= ((int64_t)1 << 30)) range *= 2;
    h->range = (int)std::min<int64_t>(range, INT32_MAX);
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, df_rho_kernel, 32 * DF_WARPS, 0);
    h->blocks_rho = sm * std::max(1, occ);
    occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, df_j_kernel, 32 * DF_WARPS, 0);
    h->blocks_j = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sm * std::max(1, occ),
                                                               (npair + DF_WARPS - 1) / DF_WARPS));
    std::vector<int64_t> doff((size_t)std::max<int64_t>(npair, 1), 0);
    int64_t nabt = 0;
    for (int64_t p = 0; p < npair; p++) { doff[p] = nabt; nabt += (int64_t)desc[p].z * desc[p].w; }
    h->nab_total = nabt;
    std::vector<int> order((size_t)std::max<int64_t>(npair, 1), 0);
    for (int64_t p = 0; p < npair; p++) order[p] = (int)p;
    std::stable_sort(order.begin(), order.begin() + npair, [&](int x, int y) {
        return desc[x].z * desc[x].w > desc[y].z * desc[y].w;
    });
    if (npair > INT32_MAX) { delete h; return df_fail("df: more than 2^31 pairs"); }
    if (cudaMalloc(&h->d_seg, sizeof(int64_t) * seg.size()) != cudaSuccess
        || cudaMalloc(&h->d_desc, sizeof(int4) * desc.size()) != cudaSuccess
        || cudaMalloc(&h->d_order, sizeof(int) * order.size()) != cudaSuccess
        || cudaMalloc(&h->d_counter, sizeof(unsigned long long)) != cudaSuccess
        || cudaMalloc(&h->d_doff, sizeof(int64_t) * doff.size()) != cudaSuccess
        || cudaMalloc(&h->d_dw, sizeof(double) * std::max<int64_t>(nabt, 1)) != cudaSuccess
        || cudaMemcpy(h->d_doff, doff.data(), sizeof(int64_t) * doff.size(), cudaMemcpyHostToDevice) != cudaSuccess
        || cudaMemcpy(h->d_seg, seg.data(), sizeof(int64_t) * seg.size(), cudaMemcpyHostToDevice) != cudaSuccess
        || cudaMemcpy(h->d_desc, desc.data(), sizeof(int4) * desc.size(), cudaMemcpyHostToDevice) != cudaSuccess
        || cudaMemcpy(h->d_order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(h->d_seg);
        cudaFree(h->d_desc);
        cudaFree(h->d_order);
        cudaFree(h->d_counter);
        cudaFree(h->d_doff);
        cudaFree(h->d_dw);
        delete h;
        cg_set_error_msg("df: device allocation or copy failed");
        return CINTGPU_ERR_NOMEM;
    }
    *out = h;
    return 0;
}

int64_t cintgpu_df_size(const CINTGPUDF *df) { return df ? df->size : -1; }

int cintgpu_df_rho(CINTGPUDF *df, const double *T, const double *dm, double *rho, void *stream)
{
    if (!df || (!T && df->size) || !dm || !rho) return df_fail("df_rho: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(rho, 0, sizeof(double) * df->naux, st) != cudaSuccess) {
        cg_set_error_msg("df_rho: memset failed");
        return CINTGPU_ERR_CUDA;
    }
    if (df->npair == 0) return 0;
    df_density_kernel<<<df->blocks_j, 32 * DF_WARPS, 0, st>>>(df->d_desc, df->d_doff, df->npair, dm, df->nao,
                                                              df->d_dw);
    df_rho_kernel<<<df->blocks_rho, 32 * DF_WARPS, 0, st>>>(T, df->d_seg, df->d_desc, df->npair, df->range,
                                                            df->naux, df->d_doff, df->d_dw, rho);
    if (cudaGetLastError() != cudaSuccess) { cg_set_error_msg("df_rho: launch failed"); return CINTGPU_ERR_CUDA; }
    return 0;
}

int cintgpu_df_j(CINTGPUDF *df, const double *T, const double *c, double *vj, void *stream)
{
    if (!df || (!T && df->size) || !c || !vj) return df_fail("df_j: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(vj, 0, sizeof(double) * df->nao * df->nao, st) != cudaSuccess
        || cudaMemsetAsync(df->d_counter, 0, sizeof(unsigned long long), st) != cudaSuccess) {
        cg_set_error_msg("df_j: memset failed");
        return CINTGPU_ERR_CUDA;
    }
    if (df->npair == 0) return 0;
    df_j_kernel<<<df->blocks_j, 32 * DF_WARPS, 0, st>>>(T, df->d_seg, df->d_desc, df->d_order, df->npair,
                                                        df->naux, c, df->nao, vj, df->d_counter);
    if (cudaGetLastError() != cudaSuccess) { cg_set_error_msg("df_j: launch failed"); return CINTGPU_ERR_CUDA; }
    return 0;
}

void cintgpu_df_destroy(CINTGPUDF *df)
{
    if (!df) return;
    cudaFree(df->d_seg);
    cudaFree(df->d_desc);
    cudaFree(df->d_order);
    cudaFree(df->d_counter);
    cudaFree(df->d_doff);
    cudaFree(df->d_dw);
    delete df;
}

}  // extern "C"
