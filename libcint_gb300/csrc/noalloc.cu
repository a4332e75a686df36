/*
 * Allocation-free batched int2e_sph.
 *
 * Some callers cannot allocate device memory during a call: frameworks that own the device memory
 * budget through their own allocator and forbid side allocations, or code running where a
 * cudaMalloc would synchronise the device or fail outright.  cintgpu_int2e_sph_noalloc serves
 * them: it evaluates the same kernels as cintgpu_plan_execute, but every piece of device scratch
 * (pair tables, surviving-primitive lists, task lists, Cartesian accumulators, output staging)
 * lives in one file-scope __device__ array of CINTGPU_NOALLOC_BYTES (32 MiB) that every GPU
 * loading this library holds until the process exits.  The caller passes the inputs (host
 * atm/bas/env and shell quartets) and the device output buffer.
 *
 * Set-up: the first call on a device (with that device current) looks up the array's device
 * address with cudaGetSymbolAddress and caches it for that device.  The cached address belongs to
 * the device's primary context: do not keep using the library on a device after
 * cudaDeviceReset.  All calls share the array and it keeps the last call's contents; the kernels
 * clear what must start at zero (counters, flags, accumulators) on every call.  Calls that overlap
 * on the GPU (different streams) race on the array: the caller serialises them.  The plan image
 * is copied into the array from host memory with a stream-ordered copy that returns once the
 * data is staged.
 */
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "cintgpu_internal.h"

#define CINTGPU_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) char g_noalloc_scratch[CINTGPU_NOALLOC_BYTES];

static std::mutex g_noalloc_mu;
static char *g_noalloc_addr[CINTGPU_NOALLOC_MAX_DEVICES];

/* device address of this device's copy of the array; looked up once per device */
static int noalloc_region(char **region)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= CINTGPU_NOALLOC_MAX_DEVICES) {
        cg_set_error_msg("cintgpu_int2e_sph_noalloc: no usable current device");
        return CINTGPU_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        char *a = nullptr;
        e = cudaGetSymbolAddress((void **)&a, g_noalloc_scratch);
        if (e != cudaSuccess || !a) {
            char msg[200];
            snprintf(msg, sizeof(msg), "cintgpu_int2e_sph_noalloc: cudaGetSymbolAddress failed: %s",
                     cudaGetErrorString(e));
            cg_set_error_msg(msg);
            return CINTGPU_ERR_CUDA;
        }
        g_noalloc_addr[dev] = a;
    }
    *region = g_noalloc_addr[dev];
    return 0;
}

extern "C" int cintgpu_int2e_sph_noalloc(double *out_dev, const int *shls, int64_t n,
                                         const int *atm, int natm, const int *bas, int nbas,
                                         const double *env, void *stream)
{
    int rc = cg_init();
    if (rc) return rc;
    char *region = nullptr;
    rc = noalloc_region(&region);
    if (rc) return rc;
    CINTGPUPlan *P = cg_plan_new();
    cg_plan_separate_output(P);   /* keeps the footprint inside the static array */
    int64_t split = n < (int64_t)cg_sm_count() * 16 ? (int64_t)cg_sm_count() * 8 : 0;
    rc = cg_plan_build(P, CINTGPU_INT2E_SPH, shls, n, nullptr, atm, natm, bas, nbas, env, split);
    if (!rc) {
        size_t need = cg_plan_bytes(P);
        if (need > (size_t)CINTGPU_NOALLOC_BYTES) {
            char msg[240];
            snprintf(msg, sizeof(msg),
                     "cintgpu_int2e_sph_noalloc: this batch needs %zu bytes of device scratch; the "
                     "allocation-free entry point is limited to %d bytes (split the batch or use "
                     "cintgpu_plan_create)", need, (int)CINTGPU_NOALLOC_BYTES);
            cg_set_error_msg(msg);
            rc = CINTGPU_ERR_NOMEM;
        }
    }
    if (!rc) rc = cg_plan_place(P, region, (size_t)CINTGPU_NOALLOC_BYTES, (cudaStream_t)stream);
    if (!rc) rc = cg_plan_run(P, out_dev, (cudaStream_t)stream);
    cg_plan_free_host(P);
    return rc;
}
