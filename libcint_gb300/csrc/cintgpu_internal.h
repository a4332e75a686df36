/* Host-side planner hooks shared between translation units of libcintgpu (not exported). */
#ifndef CINTGPU_INTERNAL_H
#define CINTGPU_INTERNAL_H
#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>
#include "cintgpu.h"

int cg_init(void);
int cg_sm_count(void);
void cg_set_error_msg(const char *msg);
CINTGPUPlan *cg_plan_new(void);
void cg_plan_free_host(CINTGPUPlan *P);
int cg_plan_build(CINTGPUPlan *P, int kind, const int *shls, int64_t n, const int64_t *offsets,
                  const int *atm, int natm, const int *bas, int nbas, const double *env,
                  int64_t split_target);
/* transform outputs in a separate kernel instead of inside the integral kernel (smaller device
 * footprint: no per-warp transform scratch for the integral kernel's warps) */
void cg_plan_separate_output(CINTGPUPlan *P);
size_t cg_plan_bytes(const CINTGPUPlan *P);
/* lay the plan out in a caller-owned device region and copy its host images there
 * (stream-ordered, from pageable memory); allocates no device memory */
int cg_plan_place(CINTGPUPlan *P, char *region, size_t region_bytes, cudaStream_t stream);
int cg_plan_run(CINTGPUPlan *P, double *out_dev, cudaStream_t stream);
extern "C" int cg_eri_tables(int li, int lj, int lk, int ll, int bra, int *info, int *groups,
                             int maxg, int *perm, int maxp, int *prog, int maxprog, int *rounds,
                             int maxr);
#endif
