// FP64 (DFMA), FP64 tensor-core (DMMA) and FP32 (FFMA) issue-rate microbenchmark: the denominator
// of the roofline that bench.py reports for the Rys kernels (they are FP64-issue bound), and the
// evidence for keeping their contractions off the FP64 tensor cores.  8 independent chains per
// thread (DFMA, FFMA) or 4 independent accumulator tiles per warp (DMMA m8n8k4, 512 flops per
// warp-wide instruction), grids of 1-2 blocks per SM, CUDA events around one launch after a
// warm-up launch.  Run by `python bench.py --only fp64peak`, which builds it with
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o <tmp>/fp64_peak bench_fp64_peak.cu
#include <cstdio>
#include <cuda_runtime.h>
// D = A B + C on the FP64 tensor cores, one 8x8x4 tile per warp instruction (mma.sync, f64)
__device__ __forceinline__ void dmma_8x8x4(double &d0, double &d1, double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                 : "+d"(d0), "+d"(d1) : "d"(a), "d"(b));
}
__global__ void dmma_kernel(double *out, int iters, double a, double b)
{
    double c[4][2];
#pragma unroll
    for (int t = 0; t < 4; t++) { c[t][0] = threadIdx.x * 1e-3 + t; c[t][1] = 0.5 * t; }
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int t = 0; t < 4; t++) dmma_8x8x4(c[t][0], c[t][1], a, b);
    }
    double s = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) s += c[t][0] + c[t][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template<int NCHAIN>
__global__ void dfma_kernel(double *out, int iters, double a, double b) {
    double acc[NCHAIN];
#pragma unroll
    for (int c = 0; c < NCHAIN; c++) acc[c] = threadIdx.x * 1e-3 + c;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < NCHAIN; c++) acc[c] = fma(acc[c], a, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < NCHAIN; c++) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
// the same chains on the first `active` lanes of every warp only: whether a partially active
// warp instruction costs the FP64 pipe the time of a full one
template<int NCHAIN>
__global__ void dfma_lanes_kernel(double *out, int iters, double a, double b, int active) {
    double s = 0;
    if ((int)(threadIdx.x & 31) < active) {
        double acc[NCHAIN];
#pragma unroll
        for (int c = 0; c < NCHAIN; c++) acc[c] = threadIdx.x * 1e-3 + c;
        for (int i = 0; i < iters; i++) {
#pragma unroll
            for (int c = 0; c < NCHAIN; c++) acc[c] = fma(acc[c], a, b);
        }
#pragma unroll
        for (int c = 0; c < NCHAIN; c++) s += acc[c];
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template<int NCHAIN>
__global__ void ffma_kernel(float *out, int iters, float a, float b) {
    float acc[NCHAIN];
#pragma unroll
    for (int c = 0; c < NCHAIN; c++) acc[c] = threadIdx.x * 1e-3f + c;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < NCHAIN; c++) acc[c] = fmaf(acc[c], a, b);
    }
    float s = 0;
#pragma unroll
    for (int c = 0; c < NCHAIN; c++) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
int main() {
    int dev = 0; cudaDeviceProp p; cudaGetDeviceProperties(&p, dev);
    printf("name=%s sms=%d cc=%d.%d smem/block optin=%zu regs/sm=%d l2=%d\n", p.name, p.multiProcessorCount,
           p.major, p.minor, p.sharedMemPerBlockOptin, p.regsPerMultiprocessor, p.l2CacheSize);
    int sms = p.multiProcessorCount;
    double *dout; cudaMalloc(&dout, sizeof(double) * sms * 16 * 1024);
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    int cfgs[][2] = {{128, 1}, {256, 1}, {256, 2}, {512, 2}, {1024, 2}, {32, 1}, {64,1}};
    for (auto &c : cfgs) {
        int threads = c[0], bps = c[1];
        int blocks = sms * bps;
        int iters = 20000;
        dfma_kernel<8><<<blocks, threads>>>(dout, 100, 0.999, 1e-3);
        cudaEventRecord(e0);
        dfma_kernel<8><<<blocks, threads>>>(dout, iters, 0.999, 1e-3);
        cudaEventRecord(e1); cudaEventSynchronize(e1);
        float ms; cudaEventElapsedTime(&ms, e0, e1);
        double flops = 2.0 * 8 * iters * (double)blocks * threads;
        printf("DFMA threads=%d blocks/sm=%d : %.3f ms  %.3f TFLOP/s\n", threads, bps, ms, flops / ms / 1e9);
    }
    for (auto &c : cfgs) {
        int threads = c[0], bps = c[1];
        int blocks = sms * bps;
        int iters = 20000;
        dmma_kernel<<<blocks, threads>>>(dout, 100, 1e-3, 0.999);
        cudaEventRecord(e0);
        dmma_kernel<<<blocks, threads>>>(dout, iters, 1e-3, 0.999);
        cudaEventRecord(e1); cudaEventSynchronize(e1);
        float ms; cudaEventElapsedTime(&ms, e0, e1);
        double flops = 512.0 * 4 * iters * (double)blocks * (threads / 32);
        printf("DMMA threads=%d blocks/sm=%d : %.3f ms  %.3f TFLOP/s\n", threads, bps, ms, flops / ms / 1e9);
    }
    {
        const int threads = 256, blocks = sms * 2, iters = 20000;
        const int lanes[] = {32, 16, 8, 4, 1};
        for (int k : lanes) {
            dfma_lanes_kernel<8><<<blocks, threads>>>(dout, 100, 0.999, 1e-3, k);
            cudaEventRecord(e0);
            dfma_lanes_kernel<8><<<blocks, threads>>>(dout, iters, 0.999, 1e-3, k);
            cudaEventRecord(e1); cudaEventSynchronize(e1);
            float ms; cudaEventElapsedTime(&ms, e0, e1);
            double warp_instr = 8.0 * iters * (double)blocks * (threads / 32);
            printf("DFMA-lanes active=%d threads=%d blocks/sm=2 : %.3f ms  %.3f G warp-instr/s\n", k, threads,
                   ms, warp_instr / ms / 1e6);
        }
    }
    float *fout = (float*)dout;
    for (auto &c : cfgs) {
        int threads = c[0], bps = c[1];
        int blocks = sms * bps;
        int iters = 20000;
        ffma_kernel<8><<<blocks, threads>>>(fout, 100, 0.999f, 1e-3f);
        cudaEventRecord(e0);
        ffma_kernel<8><<<blocks, threads>>>(fout, iters, 0.999f, 1e-3f);
        cudaEventRecord(e1); cudaEventSynchronize(e1);
        float ms; cudaEventElapsedTime(&ms, e0, e1);
        double flops = 2.0 * 8 * iters * (double)blocks * threads;
        printf("FFMA threads=%d blocks/sm=%d : %.3f ms  %.3f TFLOP/s\n", threads, bps, ms, flops / ms / 1e9);
    }
    cudaError_t err = cudaGetLastError();
    printf("err=%s\n", cudaGetErrorString(err));
    return err != cudaSuccess;
}
