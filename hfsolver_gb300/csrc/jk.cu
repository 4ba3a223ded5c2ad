// Fock two-electron part G = J - K/2 from the packed integrals.
//
// Replaces formG/formG2 (src/scf.f90:26-58), G(i,j) = sum_kl P(k,l) TT(k,l,i,j)
// with TT(k,l,i,j) = (ij|kl) - (il|kj)/2, without the dense n^4 TT the
// reference precomputes (src/scf.f90:79-105): each unique integral of the
// 8-fold packed array is read once from HBM and scattered.
//
// For a unique v = (ij|kl), i>=j, k>=l, ij>=kl, let w = v f with
// f = 1/2 per coincidence (i==j, k==l, ij==kl).  Summing the integral's 8
// index permutations gives G = Gh + Gh^T with the half-matrix updates
//   Gh[i][j] += 2 w P_kl,  Gh[k][l] += 2 w P_ij,
//   Gh[i][k] -= w P_jl/2,  Gh[j][k] -= w P_il/2,  Gh[i][l] -= w P_jk/2,  Gh[j][l] -= w P_ik/2.
// (With J and K kept apart: J = Jh + Jh^T from the first two updates and
// K = Kh + Kh^T from the last four without the -1/2.)
// A warp walks one row ij of the packed matrix (contiguous kl), so reads are
// coalesced; the row's Gh[i][j] term is reduced in the warp before one atomic.
#include "internal.h"

namespace hfgpu {

// SEPARATE: the Coulomb half-matrix goes to Gh and the exchange one (without the
// -1/2 and with the opposite sign convention, K = Kh + Kh^T) to Kh.
template <bool SEPARATE>
__global__ void jk_packed_kernel(int n, int64_t m, const double* __restrict__ ints, const double* __restrict__ P,
                                 const int2* __restrict__ pairs, double* Gh, double* Kh)
{
    double* X = SEPARATE ? Kh : Gh;
    const double kf = SEPARATE ? 1.0 : -0.5;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t ij = warp; ij < m; ij += nwarps) {
        const int2 pij = pairs[ij];
        const int i = pij.x, j = pij.y;
        const double fij = (i == j) ? 0.5 : 1.0;
        const double Pij = P[i + (int64_t)j * n];
        const double* row = ints + ij * (ij + 1) / 2;
        double gij = 0.0;
        for (int64_t kl = lane; kl <= ij; kl += 32) {
            const double v = row[kl];
            // screened-out quartets contribute nothing (integer test: keeps the FP64 pipe free)
            if ((__double_as_longlong(v) << 1) == 0) continue;
            const int2 pkl = pairs[kl];
            const int k = pkl.x, l = pkl.y;
            double w = v * fij;
            if (k == l) w *= 0.5;
            if (kl == ij) w *= 0.5;
            gij = fma(2.0 * w, P[k + (int64_t)l * n], gij);
            atomicAdd(&Gh[k + (int64_t)l * n], 2.0 * w * Pij);
            const double hw = kf * w;
            atomicAdd(&X[i + (int64_t)k * n], hw * P[j + (int64_t)l * n]);
            atomicAdd(&X[j + (int64_t)k * n], hw * P[i + (int64_t)l * n]);
            atomicAdd(&X[i + (int64_t)l * n], hw * P[j + (int64_t)k * n]);
            atomicAdd(&X[j + (int64_t)l * n], hw * P[i + (int64_t)k * n]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) gij += __shfl_xor_sync(0xffffffffu, gij, o);
        if (lane == 0) atomicAdd(&Gh[i + (int64_t)j * n], gij);
    }
}

__global__ void symmetrize_add_kernel(int n, const double* __restrict__ Gh, double* G)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    int i = idx % n, j = idx / n;
    G[idx] = Gh[idx] + Gh[j + (int64_t)i * n];
}

struct PairTable {
    int n = -1;
    DBuf<int2> d;
};

static const int2* pair_table(Context& ctx, int n)
{
    static thread_local PairTable tab;
    if (tab.n != n || tab.d.st != ctx.stream) {
        std::vector<int2> h((size_t)n * (n + 1) / 2);
        for (int i = 0; i < n; i++)
            for (int j = 0; j <= i; j++) h[(size_t)i * (i + 1) / 2 + j] = make_int2(i, j);
        tab.d = to_device(h, ctx.stream);
        tab.n = n;
    }
    return tab.d.p;
}

void jk_separate_from_packed(Context& ctx, int n, const double* d_int2, const double* dP, double* dJ, double* dK)
{
    const int2* pairs = pair_table(ctx, n);
    const int64_t m = (int64_t)n * (n + 1) / 2, nn = (int64_t)n * n;
    DBuf<double> Jh(nn, ctx.stream), Kh(nn, ctx.stream);
    Jh.zero();
    Kh.zero();
    int blocks = (int)std::min<int64_t>((m + 7) / 8, (int64_t)ctx.num_sms * 16);
    jk_packed_kernel<true><<<blocks, 256, 0, ctx.stream>>>(n, m, d_int2, dP, pairs, Jh.p, Kh.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
    symmetrize_add_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, ctx.stream>>>(n, Jh.p, dJ);
    count_launch();
    symmetrize_add_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, ctx.stream>>>(n, Kh.p, dK);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

void jk_from_packed(Context& ctx, int n, const double* d_int2, const double* dP, double* dG)
{
    const int2* pairs = pair_table(ctx, n);
    const int64_t m = (int64_t)n * (n + 1) / 2;
    DBuf<double> Gh((size_t)n * n, ctx.stream);
    Gh.zero();
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    HF_CUDA(cudaEventRecord(e0, ctx.stream));
    int blocks = (int)std::min<int64_t>((m + 7) / 8, (int64_t)ctx.num_sms * 16);
    jk_packed_kernel<false><<<blocks, 256, 0, ctx.stream>>>(n, m, d_int2, dP, pairs, Gh.p, nullptr);
    count_launch();
    HF_CUDA(cudaGetLastError());
    int64_t nn = (int64_t)n * n;
    symmetrize_add_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, ctx.stream>>>(n, Gh.p, dG);
    count_launch();
    HF_CUDA(cudaGetLastError());
    HF_CUDA(cudaEventRecord(e1, ctx.stream));
    HF_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    ctx.stat_fock_ms += ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

}  // namespace hfgpu
