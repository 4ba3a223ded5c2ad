// Green's-function pole of one orbital from the packed MO integrals: the
// reference's find_pole_diag (src/gf.f90:15-34), the fixed-point iteration
//     E <- lam(i) + Sigma_ii(E)
// from E = lam(i) until |dE| < tolE, with the second-order self-energy of
// self_energy (src/gf.f90:124-148), j = i:
//     Sigma_ii(E) = sum_{a occ; r,s virt} (ir|as) [2 (ir|as) - (is|ar)] / (E + e_a - e_r - e_s)
//                 + sum_{a,b occ; r virt} (ia|br) [2 (ia|br) - (ib|ar)] / (E + e_r - e_a - e_b).
// The numerators and the E-independent parts of the denominators are gathered
// from the packed array once (o v^2 + o^2 v terms); each iteration is then one
// reduction kernel over them and a single value back to the host.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"
#include "scf.h"

namespace hfgpu {

__device__ __forceinline__ int64_t gf_pidx(int64_t i, int64_t j, int64_t k, int64_t l)
{
    const int64_t a = i > j ? i : j, b = i > j ? j : i;
    const int64_t c = k > l ? k : l, d = k > l ? l : k;
    const int64_t ij = a * (a + 1) / 2 + b, kl = c * (c + 1) / 2 + d;
    return ij >= kl ? ij * (ij + 1) / 2 + kl : kl * (kl + 1) / 2 + ij;
}

// terms t < o v^2: (a, r, s); then (a, b, r)
__global__ void gf_terms_kernel(int n, int o, int i, const double* __restrict__ mo, const double* __restrict__ lam,
                                double* __restrict__ num, double* __restrict__ den)
{
    const int v = n - o;
    const int64_t n1 = (int64_t)o * v * v, nt = n1 + (int64_t)o * o * v;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        if (t < n1) {
            const int a = (int)(t / ((int64_t)v * v)), r = o + (int)((t / v) % v), s = o + (int)(t % v);
            const double iras = mo[gf_pidx(i, r, a, s)], isar = mo[gf_pidx(i, s, a, r)];
            num[t] = iras * (2.0 * iras - isar);
            den[t] = lam[a] - lam[r] - lam[s];
        } else {
            const int64_t u = t - n1;
            const int a = (int)(u / ((int64_t)o * v)), b = (int)((u / v) % o), r = o + (int)(u % v);
            const double iabr = mo[gf_pidx(i, a, b, r)], ibar = mo[gf_pidx(i, b, a, r)];
            num[t] = iabr * (2.0 * iabr - ibar);
            den[t] = lam[r] - lam[a] - lam[b];
        }
    }
}

// partial[block] = sum over the block's terms of num / (E + den)
__global__ void __launch_bounds__(256) gf_sigma_kernel(int64_t nt, const double* __restrict__ num,
                                                      const double* __restrict__ den, double E,
                                                      double* __restrict__ partial)
{
    double s = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x)
        s += num[t] / (E + den[t]);
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

double find_pole_diag(Context& ctx, int n, const double* d_mo, const double* d_lam, int nocc, int i, int nscf,
                      double tolE, int* niter)
{
    HF_CHECK(nocc >= 1 && nocc < n, HFGPU_ERR_INVALID, "find_pole_diag: need 1 <= nocc < n");
    HF_CHECK(i >= 0 && i < n, HFGPU_ERR_INVALID, "find_pole_diag: orbital index out of range");
    cudaStream_t st = ctx.stream;
    const int o = nocc, v = n - nocc;
    const int64_t nt = (int64_t)o * v * v + (int64_t)o * o * v;
    DBuf<double> num((size_t)nt, st), den((size_t)nt, st);
    const unsigned gt = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nt + 255) / 256, (int64_t)ctx.num_sms * 8));
    gf_terms_kernel<<<gt, 256, 0, st>>>(n, o, i, d_mo, d_lam, num.p, den.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
    double lam_i = 0;
    HF_CUDA(cudaMemcpyAsync(&lam_i, d_lam + i, sizeof(double), cudaMemcpyDeviceToHost, st));
    const unsigned gs = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nt + 255) / 256, (int64_t)ctx.num_sms * 4));
    DBuf<double> part(gs, st);
    std::vector<double> h(gs);
    HF_CUDA(cudaStreamSynchronize(st));
    double E = lam_i;
    for (int it = 1; it <= nscf; ++it) {
        const double Eold = E;
        gf_sigma_kernel<<<gs, 256, 0, st>>>(nt, num.p, den.p, E, part.p);
        count_launch();
        HF_CUDA(cudaGetLastError());
        part.download(h.data(), gs);
        HF_CUDA(cudaStreamSynchronize(st));
        double sigma = 0;
        for (double x : h) sigma += x;
        E = lam_i + sigma;
        if (niter) *niter = it;
        if (std::fabs(E - Eold) < tolE) return E;
    }
    throw Error(HFGPU_ERR_NOT_CONVERGED,
                "Green's function SCF did not converge in " + std::to_string(nscf) + " iterations.");
}

}  // namespace hfgpu
