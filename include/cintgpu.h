/*
 * libcintgpu -- GB300-native drop-in for libcint's two-electron Rys-quadrature integrals.
 *
 * Part 1 re-exports libcint's own C ABI for the hot path with identical signatures, argument
 * meaning, return values and output layout, so a caller relinks against libcintgpu.so instead of
 * libcint.so.  Each declaration cites the libcint interface it replaces.
 *
 * Part 2 is this library's batched device API (no libcint counterpart): a plan over a list of
 * shell quartets (or triples) is built once on the host, its inputs stay resident in HBM, and
 * every execution is a fixed sequence of kernel launches on a caller stream (capturable in a
 * CUDA graph).  All entry points return 0 on success or a negative status and never abort;
 * cintgpu_last_error() returns the calling thread's last message.
 */
#ifndef CINTGPU_H
#define CINTGPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- libcint data model (libcint include/cint.h.in:10-24, 26-72, 139-152) ---------------- */
#ifndef FINT
#define FINT int
#endif
#ifndef CACHE_SIZE_T
#define CACHE_SIZE_T FINT
#endif
#define PTR_EXPCUTOFF   0
#define PTR_COMMON_ORIG 1
#define PTR_RINV_ORIG   4
#define PTR_RINV_ZETA   7
#define PTR_RANGE_OMEGA 8
#define PTR_ENV_START   20
#define CHARGE_OF       0
#define PTR_COORD       1
#define NUC_MOD_OF      2
#define PTR_ZETA        3
#define ATM_SLOTS       6
#define ATOM_OF         0
#define ANG_OF          1
#define NPRIM_OF        2
#define NCTR_OF         3
#define KAPPA_OF        4
#define PTR_EXP         5
#define PTR_COEFF       6
#define BAS_SLOTS       8

#if !defined HAVE_DEFINED_CINTOPT_H
#define HAVE_DEFINED_CINTOPT_H
typedef struct {
    double rij[3];
    double eij;
    double cceij;
} PairData;
typedef struct {
    FINT **index_xyz_array;
    FINT **non0ctr;
    FINT **sortedidx;
    FINT nbas;
    double **log_max_coeff;
    PairData **pairdata;
} CINTOpt;
#endif

/* ---- Part 1: libcint drop-in ------------------------------------------------------------- */
/* Range separation: env[PTR_RANGE_OMEGA] = omega > 0 gives every integral below with the
 * long-range Coulomb erf(omega r)/r (libcint src/g2e.c:4477-4492); omega < 0 (short range) is
 * rejected.  (ij|kl), real spherical; libcint src/cint2e.c:1186-1194, include/cint_funcs.h:20-23 */
CACHE_SIZE_T int2e_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                       FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
/* (ij|kl), Cartesian; libcint src/cint2e.c:1202-1210 */
CACHE_SIZE_T int2e_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                        FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
/* optimizer; libcint src/cint2e.c:1195-1200 */
void int2e_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
/* (nabla i j|kl), 3 components; libcint src/autocode/grad2.c:69-88, include/cint_funcs.h:680-683 */
CACHE_SIZE_T int2e_ip1_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                           FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
CACHE_SIZE_T int2e_ip1_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                            FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
void int2e_ip1_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
/* (ij|nabla k l), 3 components; libcint src/autocode/grad2.c:163-176 (ng = {0,0,1,0,...}) */
CACHE_SIZE_T int2e_ip2_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                           FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
CACHE_SIZE_T int2e_ip2_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                            FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
void int2e_ip2_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
/* (nabla nabla i j|kl), 9 components (xx, xy, xz, yx, ..., zz); libcint
 * src/autocode/hess.c:1175-1194 (ng = {2,0,0,0,...}) */
CACHE_SIZE_T int2e_ipip1_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                             FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
CACHE_SIZE_T int2e_ipip1_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                              FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
void int2e_ipip1_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
/* (nabla i j|k) and (ij|nabla k), 3 components each; libcint src/autocode/int3c2e.c:72-87 and
 * :153-168 */
CACHE_SIZE_T int3c2e_ip1_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                             FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
CACHE_SIZE_T int3c2e_ip1_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                              FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
void int3c2e_ip1_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
CACHE_SIZE_T int3c2e_ip2_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                             FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
CACHE_SIZE_T int3c2e_ip2_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                              FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
void int3c2e_ip2_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
/* (ij|k), real spherical / Cartesian; libcint src/cint3c2e.c:693-717 */
CACHE_SIZE_T int3c2e_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                         FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
CACHE_SIZE_T int3c2e_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                          FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
void int3c2e_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
/* (i|k), the density-fitting metric, real spherical / Cartesian; libcint src/cint2c2e.c:351-375
 * (dims holds 2 entries) */
CACHE_SIZE_T int2c2e_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                         FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
CACHE_SIZE_T int2c2e_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                          FINT *bas, FINT nbas, double *env, CINTOpt *opt, double *cache);
void int2c2e_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
/* libcint src/optimizer.c:40-72 */
void CINTdel_2e_optimizer(CINTOpt **opt);
void CINTdel_optimizer(CINTOpt **opt);

/* CINT2 8-argument wrappers; libcint src/misc.h:34-60 (ALL_CINT) */
FINT cint2e_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                double *env, CINTOpt *opt);
FINT cint2e_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                 double *env, CINTOpt *opt);
void cint2e_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
void cint2e_cart_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env);
FINT cint2e_ip1_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                    double *env, CINTOpt *opt);
FINT cint2e_ip1_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                     double *env, CINTOpt *opt);
void cint2e_ip1_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                              double *env);
FINT cint2e_ip2_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                    double *env, CINTOpt *opt);
FINT cint2e_ip2_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                     double *env, CINTOpt *opt);
void cint2e_ip2_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                              double *env);
FINT cint2e_ipip1_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                      double *env, CINTOpt *opt);
FINT cint2e_ipip1_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                       double *env, CINTOpt *opt);
void cint2e_ipip1_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                                double *env);
FINT cint3c2e_ip1_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                      double *env, CINTOpt *opt);
FINT cint3c2e_ip1_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                       double *env, CINTOpt *opt);
FINT cint3c2e_ip2_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                      double *env, CINTOpt *opt);
FINT cint3c2e_ip2_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                       double *env, CINTOpt *opt);
FINT cint3c2e_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                  double *env, CINTOpt *opt);
FINT cint3c2e_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                   double *env, CINTOpt *opt);
void cint3c2e_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                            double *env);
FINT cint2c2e_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                  double *env, CINTOpt *opt);
FINT cint2c2e_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                   double *env, CINTOpt *opt);
void cint2c2e_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas,
                            double *env);

/* basis helpers; libcint src/misc.c:86-93, src/cint_bas.c:25-147 */
double CINTgto_norm(FINT n, double a);
FINT CINTlen_cart(const FINT l);
FINT CINTcgto_cart(const FINT bas_id, const FINT *bas);
FINT CINTcgto_spheric(const FINT bas_id, const FINT *bas);
FINT CINTtot_cgto_cart(const FINT *bas, const FINT nbas);
FINT CINTtot_cgto_spheric(const FINT *bas, const FINT nbas);
void CINTshells_cart_offset(FINT ao_loc[], const FINT *bas, const FINT nbas);
void CINTshells_spheric_offset(FINT ao_loc[], const FINT *bas, const FINT nbas);

/* ---- Part 2: batched device API (no libcint counterpart) -------------------------------- */
#define CINTGPU_INT2E_SPH      1
#define CINTGPU_INT2E_CART     2
#define CINTGPU_INT2E_IP1_SPH  3
#define CINTGPU_INT2E_IP1_CART 4
#define CINTGPU_INT3C2E_SPH    5
#define CINTGPU_INT3C2E_CART   6
#define CINTGPU_INT2C2E_SPH    12
#define CINTGPU_INT2C2E_CART   13
#define CINTGPU_INT2E_IP2_SPH  14   /* (ij|nabla k l), 3 components */
#define CINTGPU_INT2E_IP2_CART 15
#define CINTGPU_INT3C2E_IP1_SPH  16 /* (nabla i j|k), 3 components */
#define CINTGPU_INT3C2E_IP1_CART 17
#define CINTGPU_INT3C2E_IP2_SPH  18 /* (ij|nabla k), 3 components */
#define CINTGPU_INT3C2E_IP2_CART 19
#define CINTGPU_INT2E_IPIP1_SPH  20 /* (nabla nabla i j|kl), 9 components */
#define CINTGPU_INT2E_IPIP1_CART 21

#define CINTGPU_OK              0
#define CINTGPU_ERR_ARG        -1   /* invalid argument (shell index, l, nprim, omega != 0) */
#define CINTGPU_ERR_CUDA       -2   /* a CUDA call failed */
#define CINTGPU_ERR_UNSUPPORTED -3  /* class beyond the kernels' limits */
#define CINTGPU_ERR_NOMEM      -4

/* Coulomb-like contraction and its adjoint over a list of unique shell quartets
 * (i >= j, k >= l, ij >= kl; each counted with its permutation multiplicity).  Densities and J
 * live in the plan's Cartesian AO basis (cintgpu_plan_nao_cart functions, shell order, each
 * contraction column contiguous); cintgpu_cart2sph gives the per-l transformation. */
#define CINTGPU_J_BUILD        7   /* J[ij] += sum_kl (ij|kl) D[kl] over the list */
#define CINTGPU_J_GRAD         8   /* adjoint: dL/dR for L = 1/2 sum D (ij|kl) D */
#define CINTGPU_J_GRAD_EXP     9   /* adjoint: dL/dR and dL/d(primitive exponent) */
#define CINTGPU_K_BUILD        10  /* K[ik] += sum_jl (ij|kl) D[jl] over the list (exchange) */
#define CINTGPU_JK_BUILD       11  /* J and K from one evaluation of each quartet */

/* A plan is created once and may be executed any number of times, on any stream, but by one
 * thread at a time: an execution records its arguments (density, outputs) and timing events in
 * the plan.  Different plans are independent. */
typedef struct CINTGPUPlan CINTGPUPlan;

/* Build a plan for n items (4 shell indices each, 3 for int3c2e, 2 for int2c2e) of one kind.
 * offsets[q] (may be NULL) is the element offset of item q's dense block in the output of one
 * component; NULL packs the blocks back to back in item order.  The plan copies everything it
 * needs; atm/bas/env may be freed afterwards. */
int cintgpu_plan_create(CINTGPUPlan **plan, int kind, const int *shls, int64_t n,
                        const int64_t *offsets, const int *atm, int natm, const int *bas,
                        int nbas, const double *env);
/* The same with the launch parameters an autotuner picks (no libcint counterpart): ws_kb = shared
 * memory per warp of the regular task group in KB, 8..48 (it fixes the terms per batch of every
 * class and the CTAs per SM; 0 = the default 24 or CINTGPU_WS_KB), separate_output = 1 to
 * transform outputs in their own kernel instead of at the integral kernel's tail (0 = default). */
int cintgpu_plan_create_tuned(CINTGPUPlan **plan, int kind, const int *shls, int64_t n,
                              const int64_t *offsets, const int *atm, int natm, const int *bas,
                              int nbas, const double *env, int ws_kb, int separate_output);
/* ... and per class: the nwide classes in `wide` (keys ((li*8 + lj)*8 + lk)*8 + ll in kernel order:
 * li >= lj, lk >= ll, (li, lj) >= (lk, ll); int3c2e ll = 0) run in the 48 KB-per-warp task group
 * (more terms per batch, fewer warps per SM) instead of the regular one. */
int cintgpu_plan_create_classes(CINTGPUPlan **plan, int kind, const int *shls, int64_t n,
                                const int64_t *offsets, const int *atm, int natm, const int *bas,
                                int nbas, const double *env, int ws_kb, int separate_output,
                                const int *wide, int nwide);
/* doubles per component of the output (max offset + block), and the component count */
int64_t cintgpu_plan_output_size(const CINTGPUPlan *plan);
int cintgpu_plan_ncomp(const CINTGPUPlan *plan);
/* FP64 flops of one execution by the algorithmic model of this implementation (sum over
 * surviving primitive quartets; int2e/int3c2e: VRR per term, grouped (e0|f0) accumulation) */
double cintgpu_plan_flops(const CINTGPUPlan *plan);
/* the same quartets counted with libcint's per-primitive algorithm (roots setup, VRR, HRR and
 * gout per primitive quartet, src/g2e.c:272-693 and src/cint2e.c:961-1183); int2e/int3c2e kinds,
 * 0 otherwise.  No libcint counterpart (measurement aid). */
double cintgpu_plan_flops_libcint(const CINTGPUPlan *plan);
int64_t cintgpu_plan_prim_quartets(const CINTGPUPlan *plan);
/* Launch the plan on `stream` (a cudaStream_t; NULL = legacy default stream) writing
 * out_dev[comp * output_size + offsets[q] + ...].  Asynchronous; enqueue only. */
int cintgpu_plan_execute(CINTGPUPlan *plan, double *out_dev, void *stream);
/* bytes the plan keeps resident in HBM (pair tables, task lists) and uploaded at creation */
int64_t cintgpu_plan_upload_bytes(const CINTGPUPlan *plan);
/* number of kernel launches one execution enqueues */
int cintgpu_plan_launches(const CINTGPUPlan *plan);
/* milliseconds between the start of the last execution's integral kernels and their end (the
 * output transform excluded), from CUDA events recorded on the execution's stream; synchronises
 * with that point; -1 before the first execution.  No libcint counterpart (measurement aid). */
float cintgpu_plan_compute_ms(const CINTGPUPlan *plan);
/* device-side error flags of the last execution (synchronises): 0 = fine, bit0 = a task's class
 * did not fit the kernel's shared-memory layout (its contribution is missing) */
int cintgpu_plan_status(const CINTGPUPlan *plan);
/* Cartesian AO count of the plan's basis (J/adjoint kinds) */
int cintgpu_plan_nao_cart(const CINTGPUPlan *plan);
/* J kinds: vj_dev (nao_cart^2, row major) += the contraction of the listed quartets with
 * dm_dev (Cartesian, symmetric).  Only the (I >= J) shell blocks of the pair order the plan uses
 * are written; symmetrise with J = X + X^T - diag-blocks(X) (done by the Python layer). */
int cintgpu_plan_execute_j(CINTGPUPlan *plan, const double *dm_dev, double *vj_dev, void *stream);
/* J_BUILD / K_BUILD / JK_BUILD plans: vj_dev as above (J and JK kinds), and vk_dev (nao_cart^2, row
 * major; K and JK kinds) += X with K = X + X^T for the symmetric dm_dev.  The pointer a kind does
 * not use may be NULL.  No libcint counterpart: the J/K builds of direct-SCF drivers (callers of
 * int2e_sph with the 8-fold unique quartet loop) contract each block as it is computed. */
int cintgpu_plan_execute_jk(CINTGPUPlan *plan, const double *dm_dev, double *vj_dev, double *vk_dev,
                            void *stream);
/* adjoint kinds: grad_dev (natm x 3) += dL/dR; galpha_dev (sum of nprim over shells, shell
 * order; J_GRAD_EXP only, may be NULL otherwise) += dL/d(exponent) at fixed env coefficients */
int cintgpu_plan_execute_grad(CINTGPUPlan *plan, const double *dm_dev, double *grad_dev,
                              double *galpha_dev, void *stream);
/* cart -> real spherical coefficients of angular momentum l: (2l+1) x ncart row major (identity
 * for l <= 1, whose factors libcint folds into the common factor); returns the row count */
int cintgpu_cart2sph(int l, double *c);
/* after execution completed: per item 1 if any primitive quartet survived screening */
int cintgpu_plan_nonempty(const CINTGPUPlan *plan, int *flags_host);
void cintgpu_plan_destroy(CINTGPUPlan *plan);

/* Whole-molecule J / K / adjoint over the Schwarz-screened unique quartet list, which is never
 * stored (no libcint counterpart; the caller loop of libcint examples/time_c2h6.c:719-745 with the
 * per-pair bound of its optimizer's pair data, src/optimizer.c:344-425).  pairs: npair shell
 * pairs (2 ints, i >= j), q: their bounds Q_ij = sqrt(max |(ab|ab)|).  The pairs are ordered by
 * q, largest first; the quartets are (p, q) with q <= p in that order and q_p q_q >= threshold,
 * for bra positions [p_begin, p_end) (p_end < 0: all).  kind: CINTGPU_J_BUILD, K_BUILD,
 * JK_BUILD (vj_dev / vk_dev as cintgpu_plan_execute_jk) or J_GRAD, J_GRAD_EXP (grad_dev,
 * galpha_dev as cintgpu_plan_execute_grad); dm_dev is the Cartesian density.  Chunk plans are
 * built on host threads and executed as they come; the call returns when all have run, with the
 * number of quartets in *nquartets (may be NULL). */
int cintgpu_screened_run(int kind, const int *pairs, const double *q, int64_t npair,
                         double threshold, int64_t p_begin, int64_t p_end, const int *atm, int natm,
                         const int *bas, int nbas, const double *env, const double *dm_dev,
                         double *vj_dev, double *vk_dev, double *grad_dev, double *galpha_dev,
                         int64_t *nquartets);

/* the same pipeline with the blocks written straight into a device buffer (one-component kinds:
 * int2e, int3c2e, int2c2e; out_dev holds the blocks back to back, sum of their sizes); chunk plans
 * are built on host threads ahead of the GPU and run from a ring of reused device slots, so a long
 * list costs no allocation per chunk.  Synchronous: returns when every chunk has run. */
int cintgpu_batch_device(int kind, double *out_dev, const int *shls, int64_t n, const int *atm,
                         int natm, const int *bas, int nbas, const double *env);

/* one-shot host-buffer form: plan, H2D, execute, D2H into out_host (output_size*ncomp doubles) */
int cintgpu_batch_host(int kind, double *out_host, const int *shls, int64_t n,
                       const int64_t *offsets, const int *atm, int natm, const int *bas,
                       int nbas, const double *env);

/* Allocation-free batched int2e_sph (no libcint counterpart).  For callers that cannot allocate
 * device memory during a call (frameworks that own the device memory budget through their own
 * allocator).  Same result as a CINTGPU_INT2E_SPH plan with offsets = NULL: out_dev receives the
 * dense blocks of the n quartets back to back (sum of di*dj*dk*dl doubles).  All device scratch
 * lives in one static device array of CINTGPU_NOALLOC_BYTES (32 MiB, held by every GPU that loads
 * the library until exit); a batch needing more returns CINTGPU_ERR_NOMEM with a message.  The
 * first call on a device looks up the array's address (valid until a cudaDeviceReset of that
 * device).  Calls share the array: calls that overlap on the GPU race, so serialise them.
 * Asynchronous on `stream` (a cudaStream_t); calls no cudaMalloc/cudaFree. */
#define CINTGPU_NOALLOC_BYTES (32 << 20)
int cintgpu_int2e_sph_noalloc(double *out_dev, const int *shls, int64_t n, const int *atm,
                              int natm, const int *bas, int nbas, const double *env, void *stream);

/* Density-fitted Coulomb contractions (no libcint counterpart; the caller pattern of RI-J over
 * int3c2e_sph, src/cint3c2e.c, with the metric from int2c2e_sph, src/cint2c2e.c).  The packed
 * buffer T is what a CINTGPU_INT3C2E_SPH (or _CART) plan with offsets = NULL writes for the items
 * "pair p = (i, j) with every auxiliary shell, auxiliary shells in order", pairs in the order
 * given: pair p owns di*dj*naux doubles, element (a, b, Q) at a + di*(b + dj*Q).  pairs (host):
 * npair x {oi, oj, di, dj}, the AO offsets and extents of shells i and j (oi == oj only for
 * i == j; di*dj <= 256).  Device arrays: dm and vj nao x nao row-major, rho and c naux.
 *   cintgpu_df_rho:  rho_Q = sum_p w_p sum_ab T_p[ab,Q] dm[oi+a, oj+b]   (w_p = 2 if i != j)
 *   cintgpu_df_j:    vj = 0, then vj[oi+a, oj+b] = vj[oj+b, oi+a] = sum_Q T_p[ab,Q] c_Q
 * Both are asynchronous on `stream` and read T once; calls on one handle are serialised by the
 * caller (cintgpu_df_j keeps its work counter in the handle). */
typedef struct CINTGPUDF CINTGPUDF;
int cintgpu_df_create(CINTGPUDF **df, const int *pairs, int64_t npair, int nao, int naux);
int64_t cintgpu_df_size(const CINTGPUDF *df);   /* doubles of T */
int cintgpu_df_rho(CINTGPUDF *df, const double *T_dev, const double *dm_dev, double *rho_dev,
                   void *stream);
int cintgpu_df_j(CINTGPUDF *df, const double *T_dev, const double *c_dev, double *vj_dev,
                 void *stream);
void cintgpu_df_destroy(CINTGPUDF *df);

/* Rys nodes s = t^2 and weights from the device tables, for testing: xs, s, w device arrays */
int cintgpu_rys_roots_dev(int nroots, const double *xs_dev, int count, double *s_dev,
                          double *w_dev, void *stream);
int cintgpu_rys_nmax(void);

const char *cintgpu_last_error(void);
/* Number of libcint drop-in calls (int2e_sph, ..., cint2e_sph, ...) that failed since the library
 * was loaded (no libcint counterpart).  A failed call (no usable device, a CUDA error, input the
 * kernels reject) returns 0 like a screened block but fills its block with NaN, so it cannot be
 * mistaken for one; the first failure is also reported on stderr, and cintgpu_last_error() holds
 * the calling thread's message. */
int64_t cintgpu_dropin_failures(void);
int cintgpu_device_sm_count(void);

#ifdef __cplusplus
}
#endif
#endif
