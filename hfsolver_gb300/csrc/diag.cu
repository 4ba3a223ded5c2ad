// Diagnostic entry points: the device routines behind the integral and SCF
// kernels, exposed one at a time so that tests can check them directly.
//  * hfgpu_boys: the Boys function F_0..F_M(T) exactly as the ERI kernels
//    evaluate it (boys.cuh), for comparison with the reference's Fm.
//  * hfgpu_grid_barrier_check: the bounded grid barrier of the cooperative SP2
//    and tridiagonalisation kernels (gridsync.cuh) with a caller-set time
//    limit.  Launching fewer blocks than the barrier expects makes its wait run
//    out: every block then returns with the error flag set, and the host
//    reports HFGPU_ERR_CUDA with the context still usable.
#include <algorithm>
#include <cmath>
#include <string>
#include <utility>

#include "boys.cuh"
#include "gridsync.cuh"
#include "internal.h"

namespace hfgpu {

template <int M>
__global__ void boys_eval_kernel(int64_t nt, const double* __restrict__ T, const double* __restrict__ tab,
                                 double* __restrict__ F)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    double f[M + 1];
    boys_scaled<M>(T[i], 1.0, 1.0, tab, f);
#pragma unroll
    for (int m = 0; m <= M; ++m) F[i * (M + 1) + m] = f[m];
}

template <int M>
static void boys_launch(Context& ctx, int64_t nt, const double* T, double* F)
{
    const unsigned blocks = (unsigned)((nt + 127) / 128);
    boys_eval_kernel<M><<<blocks, 128, 0, ctx.stream>>>(nt, T, ctx.boys, F);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

using BoysLaunch = void (*)(Context&, int64_t, const double*, double*);
template <int... Ms>
static constexpr BoysLaunch boys_table_of(int m, std::integer_sequence<int, Ms...>)
{
    constexpr BoysLaunch t[] = {&boys_launch<Ms>...};
    return t[m];
}

__global__ void barrier_check_kernel(unsigned* count, int* err, unsigned expected, uint64_t limit_ns)
{
    if (threadIdx.x == 0) grid_arrive_wait(count, err, expected, 1u, limit_ns);
}

}  // namespace hfgpu

using namespace hfgpu;

namespace {
template <class F>
int guarded(F&& f)
{
    try {
        f();
        return HFGPU_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return HFGPU_ERR_CUDA;
    }
}
}  // namespace

extern "C" int hfgpu_boys(int maxm, int64_t nt, const double* T, double* F)
{
    return guarded([&] {
        HF_CHECK(maxm >= 0 && maxm <= BOYS_MMAX, HFGPU_ERR_INVALID,
                 "hfgpu_boys: maxm must be in [0, " + std::to_string(BOYS_MMAX) + "]");
        HF_CHECK(nt >= 0, HFGPU_ERR_INVALID, "hfgpu_boys: nt < 0");
        if (nt == 0) return;
        HF_CHECK(T && F, HFGPU_ERR_INVALID, "hfgpu_boys: NULL array");
        for (int64_t i = 0; i < nt; ++i)
            HF_CHECK(std::isfinite(T[i]) && T[i] >= 0.0, HFGPU_ERR_INVALID,
                     "hfgpu_boys: T must be finite and >= 0 (src/special_functions.f90:218-221)");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> lk(ctx.call_mutex);
        DBuf<double> dT((size_t)nt, ctx.stream), dF((size_t)nt * (maxm + 1), ctx.stream);
        dT.upload(T, (size_t)nt);
        boys_table_of(maxm, std::make_integer_sequence<int, BOYS_MMAX + 1>{})(ctx, nt, dT.p, dF.p);
        dF.download(F, (size_t)nt * (maxm + 1));
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
    });
}

extern "C" int hfgpu_grid_barrier_check(int launched_blocks, int expected_blocks, double limit_ms,
                                        double* elapsed_ms)
{
    return guarded([&] {
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> lk(ctx.call_mutex);
        HF_CHECK(launched_blocks >= 1 && launched_blocks <= ctx.num_sms, HFGPU_ERR_INVALID,
                 "hfgpu_grid_barrier_check: launched_blocks must be in [1, number of SMs] (one block per SM is "
                 "always co-resident)");
        HF_CHECK(expected_blocks >= 1, HFGPU_ERR_INVALID, "hfgpu_grid_barrier_check: expected_blocks < 1");
        HF_CHECK(limit_ms > 0 && limit_ms <= 2000.0, HFGPU_ERR_INVALID,
                 "hfgpu_grid_barrier_check: limit_ms must be in (0, 2000]");
        DBuf<unsigned> cnt(1, ctx.stream);
        DBuf<int> err(1, ctx.stream);
        cnt.zero();
        err.zero();
        cudaEvent_t e0, e1;
        HF_CUDA(cudaEventCreate(&e0));
        HF_CUDA(cudaEventCreate(&e1));
        HF_CUDA(cudaEventRecord(e0, ctx.stream));
        barrier_check_kernel<<<launched_blocks, 32, 0, ctx.stream>>>(cnt.p, err.p, (unsigned)expected_blocks,
                                                                    (uint64_t)(limit_ms * 1e6));
        count_launch();
        HF_CUDA(cudaGetLastError());
        HF_CUDA(cudaEventRecord(e1, ctx.stream));
        int herr = 0;
        HF_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
        float ms = 0;
        HF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (elapsed_ms) *elapsed_ms = ms;
        HF_CHECK(herr == 0, HFGPU_ERR_CUDA,
                 "grid barrier timed out after " + std::to_string(limit_ms) + " ms (" +
                     std::to_string(launched_blocks) + " of " + std::to_string(expected_blocks) + " blocks arrived)");
    });
}
