// FP32 FMA throughput probe: the FP32 roofline denominator measured on the device in use.
#include <string>

#include <cuda_runtime.h>

#include "engine.hpp"
#include "mcg.h"

namespace mcg {

// 8 independent FMA chains per thread; the result is stored so nothing is optimised away.
__global__ void __launch_bounds__(256) k_ffma_probe(float* out, int iters, float x, float y) {
    float a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            a0 = fmaf(a0, x, y); a1 = fmaf(a1, x, y); a2 = fmaf(a2, x, y); a3 = fmaf(a3, x, y);
            a4 = fmaf(a4, x, y); a5 = fmaf(a5, x, y); a6 = fmaf(a6, x, y); a7 = fmaf(a7, x, y);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace mcg

extern "C" int mcg_probe_fp32_tflops(double* tflops) {
    using namespace mcg;
    if (!tflops) return fail(MCG_EINVAL, "null argument");
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(MCG_ECUDA, "no CUDA device available");
    const int blocks = sms * 8, threads = 256, iters = 2048;
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) return fail(MCG_ECUDA, "cudaMalloc failed");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_ffma_probe<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);  // warm-up
    cudaEventRecord(e0);
    k_ffma_probe<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("probe: ") + cudaGetErrorString(e));
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return MCG_OK;
}
