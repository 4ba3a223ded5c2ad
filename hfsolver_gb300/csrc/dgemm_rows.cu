// Plain FP64 AO -> MO transform: the drop-in beside the tensor-core path.
//
// The same (ia|jb) as the mixed-precision transform (mp2_mixed.cu), in the same
// half-transform order over mu >= nu pairs, with every contraction an FP64
// GEMM whose A rows are gathered straight from where the transform keeps them
// (gather_rows.cuh): the packed AO integrals, Z transposed, or dense rows.
//   1. Y[p][j][la] = sum_si (mu nu|la si) C1[si, j]        p = pair(mu >= nu)
//   2. Z[p][j][b]  = sum_la Y[p][j][la] C2[la, b]
//   3. W[q][i][mu] = sum_nu Z[pair(mu, nu)][q] C1[nu, i]   q = (j, b)
//   4. T[q][i][a]  = sum_mu W[q][i][mu] C2[mu, a]          T[j][b][i][a] = (ia|jb)
// transform_int2 (src/mbpt.f90:11-79) forms all four quarters over the full
// n^4 index space by dot products; this order uses the (mu nu) symmetry of
// the AO integrals in steps 1-2 (half the work of a dense first quarter) and
// never unpacks them.
//
// dgemm_rows_kernel: out = A B over 128 x (8 TN) output tiles, 256 threads, K in
// chunks of 16.  Thread (tx, ty) = (lane, warp) owns rows tx + 32 i (i < 4) and
// columns ty TN .. ty TN + TN - 1, so a warp's A reads from shared memory are 32
// consecutive doubles and its B reads one broadcast address.  The gathers of
// the next K chunk are issued into registers before the current chunk's
// products.  GB300's FP64 pipe (about 2 FMAs per clock per SM) bounds it: with
// 4 TN independent accumulators per thread one warp per SM sub-partition keeps
// the pipe busy.
#include <algorithm>
#include <vector>

#include "gather_rows.cuh"
#include "internal.h"
#include "scf.h"
#include "tcgemm.h"

namespace hfgpu {

namespace {
constexpr int DG_BM = 128, DG_BK = 16, DG_TM = 4, DG_THREADS = 256;
}

// B element (k, c) at B[k sk + c sc]: column-major B has sk = 1, row-major sc = 1.
// out = alpha A B + beta out (beta = 0: out is not read).
template <class Src, int TN>
__global__ void __launch_bounds__(DG_THREADS) dgemm_rows_kernel(const Src src, const int64_t M, const int K,
                                                                const double* __restrict__ B, const int64_t sk,
                                                                const int64_t sc, const int N,
                                                                double* __restrict__ out, const OutMap om,
                                                                const double alpha, const double beta)
{
    constexpr int BN = 8 * TN;
    __shared__ double As[DG_BK][DG_BM];
    __shared__ double Bs[DG_BK][BN];
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int64_t m0 = (int64_t)blockIdx.x * DG_BM;
    const int n0 = blockIdx.y * BN;
    // loader: row lr of the tile, 8 consecutive k from lk0
    const int lr = tid & (DG_BM - 1), lk0 = (tid >> 7) * 8;
    const int64_t r = m0 + lr;
    const bool live = r < M && src.live(r);
    typename Src::Row w{};
    if (live) w = src.row(r);
    double areg[8];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = k0 + lk0 + e;
            areg[e] = (live && k < K) ? src.at(w, k) : 0.0;
        }
    };
    double acc[DG_TM][TN];
#pragma unroll
    for (int i = 0; i < DG_TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;
    fetch(0);
    for (int k0 = 0; k0 < K; k0 += DG_BK) {
        __syncthreads();  // the previous chunk's products are done with As and Bs
#pragma unroll
        for (int e = 0; e < 8; ++e) As[lk0 + e][lr] = areg[e];
        for (int idx = tid; idx < DG_BK * BN; idx += DG_THREADS) {
            // consecutive threads along B's unit-stride direction: coalesced
            const int kk = sk == 1 ? idx % DG_BK : idx / BN, c = sk == 1 ? idx / DG_BK : idx % BN;
            const int k = k0 + kk, col = n0 + c;
            Bs[kk][c] = (k < K && col < N) ? __ldg(B + k * sk + col * sc) : 0.0;
        }
        __syncthreads();
        if (k0 + DG_BK < K) fetch(k0 + DG_BK);
#pragma unroll
        for (int kk = 0; kk < DG_BK; ++kk) {
            double a[DG_TM], b[TN];
#pragma unroll
            for (int i = 0; i < DG_TM; ++i) a[i] = As[kk][tx + 32 * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = Bs[kk][ty * TN + j];
#pragma unroll
            for (int i = 0; i < DG_TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < DG_TM; ++i) {
        const int64_t rr = m0 + tx + 32 * i;
        if (rr >= M || !src.live(rr)) continue;
        const int64_t orow = src.out_row(rr);
        const int64_t base = om.R ? (orow / om.R) * (om.R * om.ld) + orow % om.R : orow * om.ld;
        const int64_t cs = om.R ? om.R : 1;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int col = n0 + ty * TN + j;
            if (col < N) {
                double* o = out + base + col * cs;
                *o = beta == 0.0 ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *o);
            }
        }
    }
}

// tile width 8 TN for N columns: the fewest padded columns, then the widest tile
static int pick_tn(int N)
{
    static const int cand[] = {10, 8, 5, 4};
    int best = cand[0];
    int64_t best_cost = INT64_MAX;
    for (int tn : cand) {
        const int64_t cost = (int64_t)(N + 8 * tn - 1) / (8 * tn) * (8 * tn);
        if (cost < best_cost) {
            best_cost = cost;
            best = tn;
        }
    }
    return best;
}

template <class Src, int TN>
static void dgemm_rows_tn(Context& ctx, const Src& src, int64_t M, int K, const double* B, int64_t sk, int64_t sc,
                          int N, double* out, OutMap om, double alpha, double beta)
{
    const int64_t bx = (M + DG_BM - 1) / DG_BM;
    const int by = (N + 8 * TN - 1) / (8 * TN);
    HF_CHECK(bx <= 0x7fffffff && by <= 65535, HFGPU_ERR_UNSUPPORTED, "FP64 transform GEMM: grid too large");
    dgemm_rows_kernel<Src, TN><<<dim3((unsigned)bx, (unsigned)by), DG_THREADS, 0, ctx.stream>>>(
        src, M, K, B, sk, sc, N, out, om, alpha, beta);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

// out (M x N, placed by om) = alpha rows of src (M x K) times B (K x N, element
// (k, c) at B[k sk + c sc]) + beta out
template <class Src>
static void dgemm_rows(Context& ctx, const Src& src, int64_t M, int K, const double* B, int64_t sk, int64_t sc,
                       int N, double* out, OutMap om, double alpha = 1.0, double beta = 0.0)
{
    if (M <= 0 || N <= 0) return;
    switch (pick_tn(N)) {
        case 10: dgemm_rows_tn<Src, 10>(ctx, src, M, K, B, sk, sc, N, out, om, alpha, beta); break;
        case 8: dgemm_rows_tn<Src, 8>(ctx, src, M, K, B, sk, sc, N, out, om, alpha, beta); break;
        case 5: dgemm_rows_tn<Src, 5>(ctx, src, M, K, B, sk, sc, N, out, om, alpha, beta); break;
        default: dgemm_rows_tn<Src, 4>(ctx, src, M, K, B, sk, sc, N, out, om, alpha, beta); break;
    }
}

void dgemm_rowmajor(Context& ctx, int64_t m, int n, int k, double alpha, const double* A, int64_t lda,
                    const double* B, int64_t ldb, double beta, double* C, int64_t ldc)
{
    const DenseRowsG rows{A, lda, nullptr};
    dgemm_rows(ctx, rows, m, k, B, ldb, 1, n, C, OutMap{0, ldc}, alpha, beta);
}

// rows per operand block (Y and W), as in the mixed transform
static const int64_t FP64_BLOCK_ROWS = 1 << 20;

void ao2mo_fp64(Context& ctx, int n, const double* d_int2, const double* C1, int n1, const double* C2, int n2,
                double* T)
{
    cudaStream_t st = ctx.stream;
    HF_CHECK(n <= 4096, HFGPU_ERR_UNSUPPORTED, "FP64 transform supports up to 4096 functions");
    const int64_t npair = (int64_t)n * (n + 1) / 2;
    std::vector<int2> hp(npair);
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= i; j++) hp[(size_t)i * (i + 1) / 2 + j] = make_int2(i, j);
    DBuf<int2> pairs = to_device(hp, st);
    const int64_t nq = (int64_t)n1 * n2;
    const int nlg = (n + 15) / 16;
    DBuf<double> Z((size_t)npair * nq, st);
    // steps 1-2 over blocks of pairs (a multiple of 8: whole row blocks of the gather)
    const int64_t pb = std::max<int64_t>(8, FP64_BLOCK_ROWS / n / 8 * 8);
    DBuf<double> Y((size_t)std::min(pb, npair) * n1 * n, st);
    for (int64_t p0 = 0; p0 < npair; p0 += pb) {
        const int64_t np = std::min(pb, npair - p0);
        const PackedRowsBlocked rows1{d_int2, pairs.p, p0, np, n, nlg, nullptr};
        dgemm_rows(ctx, rows1, (np + 7) / 8 * nlg * 128, n, C1, 1, n, n1, Y.p, OutMap{n, n1});
        ctx.trace_mark("fp64 step 1");
        const DenseRowsG rows2{Y.p, n, nullptr};
        dgemm_rows(ctx, rows2, np * n1, n, C2, 1, n, n2, Z.p + p0 * nq, OutMap{0, n2});
        ctx.trace_mark("fp64 step 2");
    }
    Y.release();
    DBuf<double> Zt((size_t)npair * nq, st);
    transpose_device(ctx, Z.p, npair, nq, Zt.p);
    Z.release();
    const int64_t qb = std::max<int64_t>(1, FP64_BLOCK_ROWS / std::max(n, n1));
    DBuf<double> W((size_t)std::min(qb, nq) * n1 * n, st);
    for (int64_t q0 = 0; q0 < nq; q0 += qb) {
        const int64_t nqb = std::min(qb, nq - q0);
        SymPairRows rows3{Zt.p + q0 * npair, npair, n};
        dgemm_rows(ctx, rows3, nqb * n, n, C1, 1, n, n1, W.p, OutMap{n, n1});
        ctx.trace_mark("fp64 step 3");
        const DenseRowsG rows4{W.p, n, nullptr};
        dgemm_rows(ctx, rows4, nqb * n1, n, C2, 1, n, n2, T + q0 * n1 * n2, OutMap{0, n2});
        ctx.trace_mark("fp64 step 4");
    }
}

}  // namespace hfgpu
