// AO -> MO transform and the MBPT2 energy, plain FP64.
//
// ao2mo_fp64 builds (i a | j b) from the packed AO integrals as four quarter
// transforms, the same contraction as transform_int2 (src/mbpt.f90:11-79):
//   X[m nu la si]  = (mu nu|la si)            unpacked, a block of mu at a time
//   X1[m nu la j]  = sum_si X C1[si, j]       cuBLAS DGEMM
//   X2[m nu j b]   = sum_la X1 C2[la, b]      batched DGEMM over (m, nu)
//   X3[i nu j b]  += sum_m C1[mu, i] X2       DGEMM, accumulated over mu blocks
//   out[i a j b]   = sum_nu C2[nu, a] X3      batched DGEMM over i
// With C1 = C_occ and C2 = C_vir it gives the (ia|jb) block MBPT2 needs; with
// C1 = C2 = C it gives every (ij|kl) for the full-transform drop-in.
// mp2_energy then evaluates term1 (src/mbpt2.f90:8-31) from (ia|jb).
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

__global__ void unpack_kernel(int n, int mu0, int bm, const double* __restrict__ ints, double* X)
{
    const int64_t n3 = (int64_t)n * n * n, total = (int64_t)bm * n3;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = e;
        const int si = (int)(r % n); r /= n;
        const int la = (int)(r % n); r /= n;
        const int nu = (int)(r % n); r /= n;
        const int mu = mu0 + (int)r;
        X[e] = ints[pidx(mu, nu, la, si)];
    }
}

void ao2mo_fp64(Context& ctx, int n, const double* d_int2, const double* C1, int n1, const double* C2, int n2,
                double* out)
{
    cudaStream_t st = ctx.stream;
    const double one = 1.0, zero = 0.0;
    const int64_t n3 = (int64_t)n * n * n;
    int bm = (int)std::max<int64_t>(1, std::min<int64_t>(n, (int64_t)500000000 / n3));
    DBuf<double> X((size_t)bm * n3, st), X1((size_t)bm * n * n * n1, st), X2((size_t)bm * n * n1 * n2, st);
    const int64_t r3 = (int64_t)n * n1 * n2;
    DBuf<double> X3((size_t)r3 * n1, st);
    for (int mu0 = 0; mu0 < n; mu0 += bm) {
        const int b = std::min(bm, n - mu0);
        unpack_kernel<<<std::max(1, ctx.num_sms * 8), 256, 0, st>>>(n, mu0, b, d_int2, X.p);
        count_launch();
        HF_CUDA(cudaGetLastError());
        HF_CUBLAS(cublasDgemm(ctx.blas, CUBLAS_OP_T, CUBLAS_OP_N, n1, b * n * n, n, &one, C1, n, X.p, n, &zero,
                              X1.p, n1));
        HF_CUBLAS(cublasDgemmStridedBatched(ctx.blas, CUBLAS_OP_T, CUBLAS_OP_T, n2, n1, n, &one, C2, n, 0, X1.p,
                                            n1, (int64_t)n1 * n, &zero, X2.p, n2, (int64_t)n1 * n2, b * n));
        const double beta = mu0 == 0 ? 0.0 : 1.0;
        HF_CUBLAS(cublasDgemm(ctx.blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)r3, n1, b, &one, X2.p, (int)r3, C1 + mu0, n,
                              &beta, X3.p, (int)r3));
    }
    HF_CUBLAS(cublasDgemmStridedBatched(ctx.blas, CUBLAS_OP_N, CUBLAS_OP_N, n1 * n2, n2, n, &one, X3.p, n1 * n2,
                                        r3, C2, n, 0, &zero, out, n1 * n2, (int64_t)n2 * n1 * n2, n1));
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
