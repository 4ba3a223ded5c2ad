// Third-order Moller-Plesset energy on the GPU, from the packed MO integrals.
//
// Same E3 as hfsolver's mbpt3 (src/mbpt.f90:161-169), the sum of the three
// terms of src/mbpt3.f90:8-128 (closed shell, all electrons correlated).  The
// reference evaluates each term as six nested loops over packed-index gathers;
// here each term is regrouped into dense FP64 GEMMs over compound indices
// (o = occupied, v = virtual, D_ab^rs = e_a + e_b - e_r - e_s):
//   term3 (mbpt3.f90:96-126) = sum_ab,rs,tu T[ab][rs] W[rs][tu] U[ab][tu]
//   term2 (mbpt3.f90:64-94)  = sum_ab,cd,rs T[ab][rs] V[ab][cd] U[cd][rs]
//       T = (ar|bs)/D_ab^rs, U = (2(ar|bs) - (as|br))/D_ab^rs,
//       W[rs][tu] = (rt|su), V[ab][cd] = (ac|bd);
//   term1 (mbpt3.f90:8-62): its eight products regroup, by their last two
//   factors, into
//       sum_{ar,bs} T1[ar][bs] (M1 (4 P1 - 2 P2) - 2 M2 P1)[ar][bs]
//                 + 2 T2[ar][bs] (M2 P2)[ar][bs]
//       T1 = (2(ar|bs) - (br|as))/D_ab^rs, T2 = ((ar|bs) - 2(br|as))/D_ab^rs,
//       M1[ar][ct] = (ar|ct), M2[ar][ct] = (ac|rt),
//       P1[ct][bs] = (bs|ct)/D_bc^st, P2[ct][bs] = (bt|cs)/D_bc^st.
// Matrices are row-major; the products run on the row-gathered FP64 GEMM of
// dgemm_rows.cu.
#include <algorithm>
#include <vector>

#include "internal.h"
#include "scf.h"

namespace hfgpu {

__device__ __forceinline__ int64_t pidx(int64_t i, int64_t j, int64_t k, int64_t l)
{
    const int64_t a = i > j ? i : j, b = i > j ? j : i;
    const int64_t c = k > l ? k : l, d = k > l ? l : k;
    const int64_t ij = a * (a + 1) / 2 + b, kl = c * (c + 1) / 2 + d;
    return ij >= kl ? ij * (ij + 1) / 2 + kl : kl * (kl + 1) / 2 + ij;
}

// T, U over [ab][rs] (o^2 x v^2)
__global__ void mp3_tu_kernel(int o, int v, const double* __restrict__ mo, const double* __restrict__ e, double* T,
                              double* U)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)o * o * v * v) return;
    const int s = (int)(idx % v), r = (int)((idx / v) % v), b = (int)((idx / v / v) % o), a = (int)(idx / v / v / o);
    const double D = e[a] + e[b] - e[o + r] - e[o + s];
    const double arbs = mo[pidx(a, o + r, b, o + s)], asbr = mo[pidx(a, o + s, b, o + r)];
    T[idx] = arbs / D;
    U[idx] = (2 * arbs - asbr) / D;
}

// rows rs0 .. rs0 + nrows of W[rs][tu] = (rt|su) (v^2 columns)
__global__ void mp3_w_kernel(int o, int v, int64_t rs0, int64_t nrows, const double* __restrict__ mo, double* W)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t v2 = (int64_t)v * v;
    if (idx >= nrows * v2) return;
    const int64_t rs = rs0 + idx / v2;
    const int u = (int)(idx % v), t = (int)((idx / v) % v), s = (int)(rs % v), r = (int)(rs / v);
    W[idx] = mo[pidx(o + r, o + t, o + s, o + u)];
}

// V[ab][cd] = (ac|bd) (o^2 x o^2)
__global__ void mp3_v_kernel(int o, const double* __restrict__ mo, double* V)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t o2 = (int64_t)o * o;
    if (idx >= o2 * o2) return;
    const int d = (int)(idx % o), c = (int)((idx / o) % o), b = (int)((idx / o2) % o), a = (int)(idx / o2 / o);
    V[idx] = mo[pidx(a, c, b, d)];
}

// the six (ov) x (ov) arrays of term1, x = (i p), y = (j q) with i, j occupied
// and p, q virtual
__global__ void mp3_ring_kernel(int o, int v, const double* __restrict__ mo, const double* __restrict__ e, double* T1,
                                double* T2, double* M1, double* M2, double* P1c, double* P1, double* P2)
{
    const int64_t ov = (int64_t)o * v;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ov * ov) return;
    const int64_t x = idx / ov, y = idx % ov;
    const int i = (int)(x / v), p = (int)(x % v), j = (int)(y / v), q = (int)(y % v);
    const double ipjq = mo[pidx(i, o + p, j, o + q)];  // (ip|jq)
    const double jpiq = mo[pidx(j, o + p, i, o + q)];  // (jp|iq)
    const double ijpq = mo[pidx(i, j, o + p, o + q)];  // (ij|pq)
    const double Dx = e[i] + e[j] - e[o + p] - e[o + q];
    // T1, T2 with a = i, r = p, b = j, s = q
    T1[idx] = (2 * ipjq - jpiq) / Dx;
    T2[idx] = (ipjq - 2 * jpiq) / Dx;
    // M1 = (ar|ct), M2 = (ac|rt) with a = i, r = p, c = j, t = q
    M1[idx] = ipjq;
    M2[idx] = ijpq;
    // P1 = (bs|ct)/D_bc^st, P2 = (bt|cs)/D_bc^st with c = i, t = p, b = j, s = q
    const double p1 = ipjq / Dx, p2 = jpiq / Dx;  // (jq|ip) = (ip|jq); (jp|iq)
    P1[idx] = p1;
    P2[idx] = p2;
    P1c[idx] = 4 * p1 - 2 * p2;
}

// C[m][n] = alpha A[m][k] B[k][n] + beta C (row-major, leading dimensions lda, ldb, ldc)
static void gemm_rm(Context& ctx, int m, int n, int k, double alpha, const double* A, int64_t lda, const double* B,
                    int64_t ldb, double beta, double* C, int64_t ldc)
{
    dgemm_rowmajor(ctx, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
static void gemm_rm(Context& ctx, int m, int n, int k, double alpha, const double* A, const double* B, double beta,
                    double* C)
{
    gemm_rm(ctx, m, n, k, alpha, A, k, B, n, beta, C, n);
}

static unsigned grid1(int64_t n) { return (unsigned)((n + 255) / 256); }

double mbpt3_packed(Context& ctx, int n, const double* d_mo, const double* d_lam, int nocc)
{
    const int o = nocc, v = n - nocc;
    if (o <= 0 || v <= 0) return 0.0;
    cudaStream_t st = ctx.stream;
    const int64_t o2 = (int64_t)o * o, v2 = (int64_t)v * v, ov = (int64_t)o * v;
    double E = 0.0;
    {
        DBuf<double> T(o2 * v2, st), U(o2 * v2, st);
        mp3_tu_kernel<<<grid1(o2 * v2), 256, 0, st>>>(o, v, d_mo, d_lam, T.p, U.p);
        count_launch();
        HF_CUDA(cudaGetLastError());
        {  // term3: W (v^4) in row blocks of at most 2^28 elements (2 GB)
            const int64_t rows = std::max<int64_t>(1, std::min<int64_t>(v2, (1ll << 28) / v2));
            DBuf<double> W(rows * v2, st), Y(o2 * v2, st);
            for (int64_t rs0 = 0; rs0 < v2; rs0 += rows) {
                const int64_t nr = std::min(rows, v2 - rs0);
                mp3_w_kernel<<<grid1(nr * v2), 256, 0, st>>>(o, v, rs0, nr, d_mo, W.p);
                count_launch();
                HF_CUDA(cudaGetLastError());
                // Y += T[:, rs0 .. rs0 + nr] W[rs0 .. rs0 + nr, :]
                gemm_rm(ctx, (int)o2, (int)v2, (int)nr, 1.0, T.p + rs0, v2, W.p, v2, rs0 == 0 ? 0.0 : 1.0, Y.p, v2);
            }
            E += device_dot(ctx, o2 * v2, Y.p, U.p);
        }
        {  // term2
            DBuf<double> V(o2 * o2, st), Z(o2 * v2, st);
            mp3_v_kernel<<<grid1(o2 * o2), 256, 0, st>>>(o, d_mo, V.p);
            count_launch();
            HF_CUDA(cudaGetLastError());
            gemm_rm(ctx, (int)o2, (int)v2, (int)o2, 1.0, V.p, U.p, 0.0, Z.p);
            E += device_dot(ctx, o2 * v2, T.p, Z.p);
        }
    }
    {  // term1
        const int64_t nn = ov * ov;
        DBuf<double> T1(nn, st), T2(nn, st), M1(nn, st), M2(nn, st), P1c(nn, st), P1(nn, st), P2(nn, st), R(nn, st);
        mp3_ring_kernel<<<grid1(nn), 256, 0, st>>>(o, v, d_mo, d_lam, T1.p, T2.p, M1.p, M2.p, P1c.p, P1.p, P2.p);
        count_launch();
        HF_CUDA(cudaGetLastError());
        gemm_rm(ctx, (int)ov, (int)ov, (int)ov, 1.0, M1.p, P1c.p, 0.0, R.p);   // M1 (4 P1 - 2 P2)
        gemm_rm(ctx, (int)ov, (int)ov, (int)ov, -2.0, M2.p, P1.p, 1.0, R.p);   //  - 2 M2 P1
        E += device_dot(ctx, nn, T1.p, R.p);
        gemm_rm(ctx, (int)ov, (int)ov, (int)ov, 1.0, M2.p, P2.p, 0.0, R.p);    // M2 P2
        E += 2.0 * device_dot(ctx, nn, T2.p, R.p);
    }
    return E;
}

}  // namespace hfgpu
