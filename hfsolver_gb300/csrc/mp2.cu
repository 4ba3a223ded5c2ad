// The MBPT2 energy and the packed-MO drop-ins, plain FP64.
//
// ao2mo_fp64 (dgemm_rows.cu) builds (i a | j b) from the packed AO integrals,
// the contraction of transform_int2 (src/mbpt.f90:11-79): with C1 = C_occ and
// C2 = C_vir the (ia|jb) block MBPT2 needs, with C1 = C2 = C every (ij|kl) for
// the full-transform drop-in.  mp2_energy then evaluates term1
// (src/mbpt2.f90:8-31) from (ia|jb).
#include <algorithm>
#include <vector>

#include "internal.h"
#include "scf.h"

namespace hfgpu {

__device__ __forceinline__ int64_t pidx(int64_t i, int64_t j, int64_t k, int64_t l)
{
    int64_t a = i > j ? i : j, b = i > j ? j : i, c = k > l ? k : l, d = k > l ? l : k;
    int64_t ij = a * (a + 1) / 2 + b, kl = c * (c + 1) / 2 + d;
    return ij >= kl ? ij * (ij + 1) / 2 + kl : kl * (kl + 1) / 2 + ij;
}

// one block per (i, j): sum_ab (ia|jb) [2 (ia|jb) - (ib|ja)] / (e_i + e_j - e_a - e_b)
__global__ void mp2_kernel(int o, int v, const double* __restrict__ iajb, const double* __restrict__ eps,
                           double* partial)
{
    const int i = blockIdx.x % o, j = blockIdx.x / o;
    const double eij = eps[i] + eps[j];
    double s = 0.0;
    for (int e = threadIdx.x; e < v * v; e += blockDim.x) {
        const int a = e / v, b = e % v;
        const double x = iajb[(((int64_t)i * v + a) * o + j) * v + b];
        const double y = iajb[(((int64_t)i * v + b) * o + j) * v + a];
        s += x * (2 * x - y) / (eij - eps[o + a] - eps[o + b]);
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

double mp2_energy(Context& ctx, int o, int v, const double* d_iajb, const double* d_eps)
{
    if (o == 0 || v == 0) return 0.0;
    DBuf<double> part((size_t)o * o, ctx.stream);
    mp2_kernel<<<o * o, 256, 0, ctx.stream>>>(o, v, d_iajb, d_eps, part.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
    std::vector<double> h((size_t)o * o);
    part.download(h.data(), h.size());
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
    double E = 0;
    for (double x : h) E += x;
    return E;
}

// ---- drop-ins on packed MO arrays ------------------------------------------

// moint2[idx(i,j,k,l)] = full[i][j][k][l] for every unique (ij|kl)
__global__ void pack_kernel(int n, int64_t total, const double* __restrict__ full, double* packed)
{
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
         p += (int64_t)gridDim.x * blockDim.x) {
        int64_t ij = (int64_t)((sqrt(8.0 * (double)p + 1.0) - 1.0) / 2.0);
        while (ij * (ij + 1) / 2 > p) --ij;
        while ((ij + 1) * (ij + 2) / 2 <= p) ++ij;
        const int64_t kl = p - ij * (ij + 1) / 2;
        int64_t i = (int64_t)((sqrt(8.0 * (double)ij + 1.0) - 1.0) / 2.0);
        while (i * (i + 1) / 2 > ij) --i;
        while ((i + 1) * (i + 2) / 2 <= ij) ++i;
        const int64_t j = ij - i * (i + 1) / 2;
        int64_t k = (int64_t)((sqrt(8.0 * (double)kl + 1.0) - 1.0) / 2.0);
        while (k * (k + 1) / 2 > kl) --k;
        while ((k + 1) * (k + 2) / 2 <= kl) ++k;
        const int64_t l = kl - k * (k + 1) / 2;
        packed[p] = full[((i * n + j) * n + k) * n + l];
    }
}

void transform_packed(Context& ctx, int n, const double* d_int2, const double* dC, double* d_mo)
{
    DBuf<double> full((size_t)n * n * n * n, ctx.stream);
    ao2mo_fp64(ctx, n, d_int2, dC, n, dC, n, full.p);
    const int64_t total = packed_size(n);
    pack_kernel<<<std::max(1, ctx.num_sms * 8), 256, 0, ctx.stream>>>(n, total, full.p, d_mo);
    count_launch();
    HF_CUDA(cudaGetLastError());
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
}

// term1 of src/mbpt2.f90:8-31 on the packed MO integrals, block per (a, b)
__global__ void mbpt2_packed_kernel(int n, int nocc, const double* __restrict__ mo, const double* __restrict__ lam,
                                    double* partial)
{
    const int a = blockIdx.x % nocc, b = blockIdx.x / nocc;
    const int v = n - nocc;
    double s = 0.0;
    for (int e = threadIdx.x; e < v * v; e += blockDim.x) {
        const int r = nocc + e / v, t = nocc + e % v;
        const double arbs = mo[pidx(a, r, b, t)];
        const double rasb = mo[pidx(r, a, t, b)];
        const double sarb = mo[pidx(t, a, r, b)];
        s += (2.0 * arbs * rasb - 1.0 * arbs * sarb) / (-lam[r] - lam[t] + lam[a] + lam[b]);
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

double mbpt2_packed(Context& ctx, int n, const double* d_mo, const double* d_lam, int nocc)
{
    if (nocc <= 0 || nocc >= n) return 0.0;
    DBuf<double> part((size_t)nocc * nocc, ctx.stream);
    mbpt2_packed_kernel<<<nocc * nocc, 256, 0, ctx.stream>>>(n, nocc, d_mo, d_lam, part.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
    std::vector<double> h((size_t)nocc * nocc);
    part.download(h.data(), h.size());
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
    double E = 0;
    for (double x : h) E += x;
    return E;
}

}  // namespace hfgpu
