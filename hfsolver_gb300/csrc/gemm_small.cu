// FP64 GEMM for the SCF's small dense matrices (n x n with n of a few hundred).
//
// At n = 200 cuBLAS' DGEMM takes ~60 us: its tiles are large enough that the
// product runs on a few dozen SMs, and FP64 is only ~2 FMAs per cycle per SM on
// this GPU.  Here a block owns an 8 x 8 tile of C and stages its 8 rows of op(A)
// and 8 columns of op(B) whole in shared memory (stride k + 1, so the dot
// products read without bank conflicts), which spreads a 200 x 200 product over
// 625 blocks and every SM.  Each output's dot product is split into two k-halves
// (128 threads, one warp per sub-partition: a warp-wide FP64 FMA holds its
// sub-partition's FP64 pipe ~64 cycles, and 64-thread blocks left two of an SM's
// four pipes with the work).  Used for m, n, k <= 512; larger products go to
// cuBLAS.
#include "internal.h"

namespace hfgpu {

namespace {

constexpr int GS_T = 8;
constexpr int GS_MAX = 512;

constexpr int GS_KS = 2;  // k-slices per output
constexpr int GS_THREADS = GS_T * GS_T * GS_KS;

template <bool TA, bool TB>
__global__ void __launch_bounds__(GS_THREADS) gemm_small_kernel(int m, int n, int k, double alpha,
                                                                const double* __restrict__ A, int lda,
                                                                const double* __restrict__ B, int ldb, double beta,
                                                                double* C, int ldc)
{
    extern __shared__ double gs_sh[];
    const int ld = k + 1;
    double* As = gs_sh;            // row r of op(A): As[r * ld + kk]
    double* Bs = gs_sh + GS_T * ld;  // column c of op(B): Bs[c * ld + kk]
    double* part = Bs + GS_T * ld;   // partial sums of the second k-half
    const int i0 = blockIdx.x * GS_T, j0 = blockIdx.y * GS_T;
    const int t = threadIdx.x;
    for (int e = t; e < GS_T * k; e += GS_THREADS) {
        // consecutive threads take consecutive addresses of A and of B
        int r, ka;
        if (TA) { ka = e % k; r = e / k; } else { r = e % GS_T; ka = e / GS_T; }
        const int i = i0 + r;
        As[r * ld + ka] = i < m ? (TA ? A[ka + (size_t)i * lda] : A[i + (size_t)ka * lda]) : 0.0;
        int c, kb;
        if (TB) { c = e % GS_T; kb = e / GS_T; } else { kb = e % k; c = e / k; }
        const int j = j0 + c;
        Bs[c * ld + kb] = j < n ? (TB ? B[j + (size_t)kb * ldb] : B[kb + (size_t)j * ldb]) : 0.0;
    }
    __syncthreads();
    const int o = t % (GS_T * GS_T), h = t / (GS_T * GS_T);  // output, k-half
    const int r = o % GS_T, c = o / GS_T;
    const int i = i0 + r, j = j0 + c;
    const double* a = As + r * ld;
    const double* b = Bs + c * ld;
    const int kh = (k + 1) / 2, k0 = h * kh, k1 = h == 0 ? kh : k;
    double s0 = 0.0, s1 = 0.0;  // two chains: half the FMA latency on the critical path
    int kk = k0;
    for (; kk + 1 < k1; kk += 2) {
        s0 = fma(a[kk], b[kk], s0);
        s1 = fma(a[kk + 1], b[kk + 1], s1);
    }
    if (kk < k1) s0 = fma(a[kk], b[kk], s0);
    if (h == 1) part[o] = s0 + s1;
    __syncthreads();
    if (h == 1 || i >= m || j >= n) return;
    const double acc = (s0 + s1) + part[o];
    double* cp = C + i + (size_t)j * ldc;
    *cp = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *cp);
}

template <bool TA, bool TB>
void launch_small(Context& ctx, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
                  double beta, double* C, int ldc)
{
    const size_t smem = (2 * (size_t)GS_T * (k + 1) + GS_T * GS_T) * sizeof(double);
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(gemm_small_kernel<TA, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)((2 * (size_t)GS_T * (GS_MAX + 1) + GS_T * GS_T) * sizeof(double)));
    });
    const dim3 grid((unsigned)((m + GS_T - 1) / GS_T), (unsigned)((n + GS_T - 1) / GS_T));
    gemm_small_kernel<TA, TB><<<grid, GS_THREADS, smem, ctx.stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

}  // namespace

void gemm(Context& ctx, bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda,
          const double* B, int ldb, double beta, double* C, int ldc)
{
    if (m <= 0 || n <= 0) return;
    if (k <= 0 || m > GS_MAX || n > GS_MAX || k > GS_MAX) {
        HF_CUBLAS(cublasDgemm(ctx.blas, ta ? CUBLAS_OP_T : CUBLAS_OP_N, tb ? CUBLAS_OP_T : CUBLAS_OP_N, m, n, k,
                              &alpha, A, lda, B, ldb, &beta, C, ldc));
        return;
    }
    if (ta && tb) launch_small<true, true>(ctx, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (ta) launch_small<true, false>(ctx, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (tb) launch_small<false, true>(ctx, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else launch_small<false, false>(ctx, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

}  // namespace hfgpu
