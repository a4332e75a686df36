/* Internal interface between the host planner and the CUDA kernels (not part of the C-ABI). */
#ifndef CINTGPU_RYS_KERNELS_H
#define CINTGPU_RYS_KERNELS_H
#include <stdint.h>
#include <cuda_runtime.h>
#include "cintgpu_types.h"

#define CG_MODE_ERI 0
#define CG_MODE_IP1 1                /* one nabla on kernel slot 0 (i): int2e_ip1, int3c2e_ip1 */
#define CG_MODE_GRAD 2               /* adjoint, nuclear-coordinate gradient */
#define CG_MODE_GRADA 3              /* adjoint, coordinates and primitive exponents */
#define CG_MODE_ERIP 4               /* int2e classes evaluated per primitive (both transfers
                                        before contraction, libcint's order): ll >= 3 */
#define CG_MODE_IP2 6                /* one nabla on kernel slot 2 (k): int2e_ip2, int3c2e_ip2 */
#define CG_MODE_ERIB 5               /* int2e / int3c2e classes with lj >= 3 and ll <= 2: the bra
                                        transfer per term (libcint's order on the bra), the ket
                                        transfer after contraction */
#define CG_MODE_GRADJ 7              /* adjoint, nuclear-coordinate gradient of the Coulomb energy,
                                        contraction first: the densities are carried through the
                                        transfers and the 2D integrals contracted axis by axis */
#define CG_MODE_GRADAJ 8             /* the same with the primitive-exponent derivatives */
#define CG_TERMW 12                  /* doubles per term record in shared memory */
#define CG_TERMW_GRAD 20             /* term record of the adjoint kernel */
#define CG_GRAD_MAXPRIM 16           /* primitives per shell supported by the exponent adjoint */
#define CG_WS_SMALL (24 * 1024 / 8)  /* doubles of shared memory per warp, default */
#define CG_WS_MAX (48 * 1024 / 8)    /* doubles of shared memory per warp, large classes */
#define CG_C2S_MAXNNZ 16
#define CG_MODE_IPIP1 9              /* two nablas on kernel slot 0 (i): int2e_ipip1 */
#define CG_IS_IP(m) ((m) == CG_MODE_IP1 || (m) == CG_MODE_IP2 || (m) == CG_MODE_IPIP1)
/* output components and g arrays per axis (g, its nabla, the second nabla) of a mode */
#define CG_NCOMP(m) ((m) == CG_MODE_IPIP1 ? 9 : (CG_IS_IP(m) ? 3 : 1))
#define CG_NG(m) ((m) == CG_MODE_IPIP1 ? 3 : (CG_IS_IP(m) ? 2 : 1))

typedef struct {
    int lic, nroots, nmax, mmax;
    int dI, dJ, dK, dL, G, ng, nf, ncomp, scr, T;
    /* adjoint shared-memory map (doubles from the warp's base): density blocks, exponent sums,
     * cotangent (when kept in shared memory), g arrays, lane scratch */
    int off_dij, off_dkl, off_aacc, off_w, off_g, off_scr;
    int gstride;              /* doubles between consecutive terms' g arrays (3 gax) */
    int gax;                  /* doubles between a term's axis arrays: odd, so the 32 lanes of
                                 stage 2 (item = 3 term + axis) start in distinct banks */
    int termw;                /* doubles per term record */
} CGLayout;

typedef struct {
    const CGTask *tasks;
    int task0, ntasks;
    const CGPair *pairs;
    const CGPrimPair *prims;
    const int *pqlist;
    double *gctr;
    int *counter;
    int *nonempty;
    int *status;
    const double *rys_coef;
    double common_base;       /* 2 pi^3 / sqrt(pi); times the s/p factors per task */
    double omega2;            /* omega^2 of the long-range Coulomb erf(omega r)/r, minus omega^2 of
                                 the short-range erfc(omega r)/r; 0: 1/r */
    double expcut;            /* libcint's expcutoff (short-range screening of primitive quartets) */
    int three;                /* int3c2e, int2c2e: the fourth shell is the unit s partner */
    int two;                  /* int2c2e: the second shell is a unit s partner as well */
    int ws_doubles;
    /* J/K contraction (ERI mode only): accumulators in a per-warp slot, contracted at task end;
     * jmode bit 0 = J into vj, bit 1 = K into vk */
    int jmode;
    double *wscratch;         /* per-warp accumulator slots */
    int64_t wscratch_stride;
    const double *dm;         /* Cartesian density, nao x nao, row major */
    double *vj;               /* J accumulator (one triangle of shell blocks, see the host) */
    double *vk;               /* K accumulator (X with K = X + X^T) */
    int nao;
    /* contraction-first tables (ERI mode) */
    const CGEriClass *eclass;
    const CGEriGroup *egroup;
    const int *eperm;
    const int *hprog;
    const int *eround;
    /* fused output: the warp that finishes a quartet's last slice transforms and stores it */
    int fuse_out;
    const CGOutTask *outs;
    int *done;                /* finished slices per output quartet */
    double *oscr;             /* per-warp transform scratch */
    int64_t oscr_stride, nf_max;
    double *wslot;            /* per-warp accumulator slot of own-slot tasks (CGTask::own_slot) */
    int64_t wslot_stride;
    double *out;
    int ncomp;
    int64_t comp_stride;
    int64_t hrr_off1, hrr_off2;   /* J mode: transfer buffers inside the warp's slot */
} CGLaunch;

typedef struct {
    const CGTask *tasks;
    int ntasks;
    const CGPair *pairs;
    const CGPrimPair *prims;
    const int *pqlist;
    int *counter;
    int *status;
    const double *rys_coef;
    double common_base;
    double omega2;            /* as CGLaunch::omega2 */
    double expcut;
    int ws_doubles;
    const double *dm;         /* Cartesian density, nao x nao */
    int nao;
    double *grad;             /* natm x 3 */
    double *galpha;           /* per global primitive (GRADA only) */
    const CGGradClass *gclass;
    const CGGradChunk *gchunk;
    const CGGradEnt *gent;
    double *wglobal;          /* per-warp cotangent slots for classes with nf > CG_W_SMEM */
    int64_t wstride;
} CGGradLaunch;

#define CG_W_SMEM 256         /* cotangent blocks up to 256 components stay in shared memory */

#ifdef __cplusplus
extern "C" {
#endif
int cg_kernels_init(const int *c2s_nnz, const int *c2s_idx, const double *c2s_val,
                    double **rys_coef_dev);
int cg_rys_nmax(void);
int cg_blocks_per_sm(int mode, int ws_doubles);
int cg_rys_deg(void);
void cg_layout(int li, int lj, int lk, int ll, int mode, int ws_doubles, CGLayout *L);
int cg_launch_eri(const CGLaunch *P, int mode, int nblocks, cudaStream_t stream);
/* idx: the output quartets to transform (NULL: all nout); scratch per warp: two cart->sph buffers
 * of nf_max doubles, then two transfer buffers of (scratch_per_warp - 2 nf_max) / 2 doubles */
int cg_launch_output(const CGOutTask *ot, const int *idx, int nout, double *gctr, const int *nonempty,
                     double *scratch, int64_t scratch_per_warp, int64_t nf_max,
                     const CGEriClass *eclass, const int *eperm, const int *hprog, int nblocks,
                     double *out, int ncomp, int64_t comp_stride, cudaStream_t stream);
int cg_grad_tu_init(const int *c2s_nnz, const int *c2s_idx, const double *c2s_val);
int cg_launch_grad(const CGGradLaunch *P, int mode, int nblocks, cudaStream_t stream);
int cg_grad_blocks_per_sm(int mode, int ws_doubles);
int cg_launch_roots(const double *xs, int count, int n, const double *coef, double *s, double *w,
                    cudaStream_t stream);
#ifdef __cplusplus
}
#endif
#endif
