// FP64 FMA throughput probe: the roofline denominator for the FP64-bound
// integral kernels (the GPU's measured peak, not a datasheet figure).
// Each thread runs 8 independent fma chains in registers; 2 flops per fma.
#include "internal.h"

namespace hfgpu {

__global__ void fp64_fma_kernel(double* out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

double probe_fp64_tflops(Context& ctx)
{
    const int threads = 256, blocks = ctx.num_sms * 8, iters = 8192;
    DBuf<double> out((size_t)blocks * threads, ctx.stream);
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    fp64_fma_kernel<<<blocks, threads, 0, ctx.stream>>>(out.p, iters, 0.9999999, 1e-7);  // warm-up
    count_launch();
    HF_CUDA(cudaEventRecord(e0, ctx.stream));
    const int reps = 5;
    for (int r = 0; r < reps; ++r) {
        fp64_fma_kernel<<<blocks, threads, 0, ctx.stream>>>(out.p, iters, 0.9999999, 1e-7);
        count_launch();
    }
    HF_CUDA(cudaEventRecord(e1, ctx.stream));
    HF_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * 8 * iters * (double)threads * blocks * reps;
    return flops / (ms * 1e-3) / 1e12;
}

}  // namespace hfgpu
