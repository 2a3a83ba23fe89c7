// Device capability probes used by the benchmark and the autotuner's cost
// model: measured FP64 fused-multiply-add throughput of this GPU.
#include <cuda_runtime.h>

#include "symgb.h"

namespace {

// Eight independent FMA chains per thread keep the FP64 pipe busy; the
// result is stored so the work cannot be removed.
__global__ void fmaChains(double* out, int iters, double a, double b) {
    double v[8];
    for (int k = 0; k < 8; ++k) v[k] = threadIdx.x * 1e-3 + k;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = __fma_rn(v[k], a, b);
    double s = 0;
    for (int k = 0; k < 8; ++k) s += v[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int symgb_measure_fp64_rate(double* flops_per_second) {
    if (!flops_per_second) return SYMGB_ERR_ARGUMENT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SYMGB_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SYMGB_ERR_CUDA;
    const int threads = 256, blocks = sms * 8, iters = 4096;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess) return SYMGB_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fmaChains<<<blocks, threads>>>(out, iters, 0.999999, 1e-9);  // warm-up
    cudaEventRecord(e0);
    for (int r = 0; r < 5; ++r) fmaChains<<<blocks, threads>>>(out, iters, 0.999999, 1e-9);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return SYMGB_ERR_CUDA;
    *flops_per_second = 5.0 * 2.0 * 8.0 * iters * (double)threads * blocks / (ms * 1e-3);
    return SYMGB_OK;
}
