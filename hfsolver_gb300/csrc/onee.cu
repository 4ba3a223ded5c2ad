// One-electron integrals S, T, V over contracted Cartesian GTOs on the GPU.
//
// Same matrices as hfsolver's getS/getT/getV (src/qc.c:6-93 over
// src/cints.c:186-307), evaluated with McMurchie-Davidson expansions:
//   S_ab = sum c_a c_b K_ab (pi/p)^{3/2} Ex^{ab}_0 Ey^{ab}_0 Ez^{ab}_0
//   T_ab from overlaps with the ket power raised/lowered by 2 (the same
//        kinetic formula as cints.c:186-210)
//   V_ab = -sum_C Z_C sum c_a c_b K_ab (2 pi/p) sum_tuv E^{ab}_{tuv} R_tuv(p, P-C)
// One thread per shell pair and chunk of nuclei (every component pair of the
// shells at once); n x n column-major like the reference.
#include <algorithm>
#include <vector>

#include "boys.cuh"
#include "internal.h"
#include "md.cuh"

namespace hfgpu {

struct ShellOne {
    const int* L;
    const int* nprim;
    const int* prim0;
    const int* coef0;
    const int* cfn0;
    const double* xyz;  // 3 per shell
    const double* alpha;
    const double* coef;
    const int* comp_fn;
};

// 1-D Hermite coefficients E[i][j][t] (Helgaker et al. eqs. 9.5.6-9.5.7) for
// i <= IA, j <= JB, with compile-time bounds so the table stays in registers
template <int IA, int JB>
__device__ __forceinline__ void e1d_ct(double (&E)[IA + 1][JB + 1][IA + JB + 1], double xpa, double xpb, double i2p)
{
#pragma unroll
    for (int i = 0; i <= IA; ++i)
#pragma unroll
        for (int j = 0; j <= JB; ++j)
#pragma unroll
            for (int t = 0; t <= IA + JB; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
#pragma unroll
    for (int i = 0; i < IA; ++i)
#pragma unroll
        for (int t = 0; t <= i + 1; ++t) {
            double v = xpa * E[i][0][t];
            if (t > 0) v = fma(i2p, E[i][0][t - 1], v);
            if (t + 1 <= i) v = fma((double)(t + 1), E[i][0][t + 1], v);
            E[i + 1][0][t] = v;
        }
#pragma unroll
    for (int i = 0; i <= IA; ++i)
#pragma unroll
        for (int j = 0; j < JB; ++j)
#pragma unroll
            for (int t = 0; t <= i + j + 1; ++t) {
                double v = xpb * E[i][j][t];
                if (t > 0) v = fma(i2p, E[i][j][t - 1], v);
                if (t + 1 <= i + j) v = fma((double)(t + 1), E[i][j][t + 1], v);
                E[i][j + 1][t] = v;
            }
}

// blockIdx.y = a chunk of ONEE_ATOMS nuclei: chunk 0 also writes S and T; every
// chunk adds its nuclei's attraction to V (zeroed by the caller) atomically.
constexpr int ONEE_ATOMS = 4;

// One thread per shell pair (A, B) of one pair type (l_A >= l_B) and chunk of
// nuclei.  The 1-D tables of a primitive pair serve every component pair, and
// the Boys values and R_tuv of a nucleus serve every component pair as well.
// A == B: only component pairs with a >= b are formed (both triangle entries
// are written from them).
template <int LA, int LB>
__global__ void __launch_bounds__(64) onee_shell_kernel(ShellOne sh, const int2* __restrict__ pairs, int npairs,
                                                        int n, int nat, const int* __restrict__ Z,
                                                        const double* __restrict__ C, const double* __restrict__ boys,
                                                        double* S, double* T, double* V)
{
    constexpr double PI = 3.14159265358979323846;
    constexpr int NA = ncart(LA), NB = ncart(LB), L = LA + LB;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= npairs) return;
    const int2 pr = pairs[idx];
    const int A = pr.x, B = pr.y;
    const double ax = sh.xyz[3 * A], ay = sh.xyz[3 * A + 1], az = sh.xyz[3 * A + 2];
    const double bx = sh.xyz[3 * B], by = sh.xyz[3 * B + 1], bz = sh.xyz[3 * B + 2];
    const double rab2 = (ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz);
    const int npa = sh.nprim[A], npb = sh.nprim[B];
    const double* alA = sh.alpha + sh.prim0[A];
    const double* alB = sh.alpha + sh.prim0[B];
    const double* coA = sh.coef + sh.coef0[A];
    const double* coB = sh.coef + sh.coef0[B];
    const bool st_chunk = blockIdx.y == 0;
    const int c0 = blockIdx.y * ONEE_ATOMS, c1 = min(nat, c0 + ONEE_ATOMS);
    double sacc[NA * NB], tacc[NA * NB], vacc[NA * NB];
#pragma unroll
    for (int k = 0; k < NA * NB; ++k) sacc[k] = tacc[k] = vacc[k] = 0.0;
    for (int pa = 0; pa < npa; ++pa)
        for (int pb = 0; pb < npb; ++pb) {
            const double a = alA[pa], b = alB[pb];
            const double p = a + b, ip = 1.0 / p;
            const double px = (a * ax + b * bx) * ip, py = (a * ay + b * by) * ip, pz = (a * az + b * bz) * ip;
            const double K = exp(-a * b * ip * rab2);
            // component coefficients c_a(pa), c_b(pb)
            double ca[NA], cb[NB];
#pragma unroll
            for (int i = 0; i < NA; ++i) ca[i] = coA[i * npa + pa];
#pragma unroll
            for (int j = 0; j < NB; ++j) cb[j] = coB[j * npb + pb];
            if (st_chunk) {
                // overlap and kinetic (cints.c:186-232 in terms of 1-D overlaps):
                // E_0 tables with the ket power raised by up to 2
                double Ex[LA + 1][LB + 3][LA + LB + 3], Ey[LA + 1][LB + 3][LA + LB + 3], Ez[LA + 1][LB + 3][LA + LB + 3];
                e1d_ct<LA, LB + 2>(Ex, px - ax, px - bx, 0.5 * ip);
                e1d_ct<LA, LB + 2>(Ey, py - ay, py - by, 0.5 * ip);
                e1d_ct<LA, LB + 2>(Ez, pz - az, pz - bz, 0.5 * ip);
                const double pre = K * PI * ip * sqrt(PI * ip);
#pragma unroll
                for (int i = 0; i < NA; ++i)
#pragma unroll
                    for (int j = 0; j < NB; ++j) {
                        const Cart c1_ = cart(LA, i), c2 = cart(LB, j);
                        const double sx = Ex[c1_.l][c2.l][0], sy = Ey[c1_.m][c2.m][0], sz = Ez[c1_.n][c2.n][0];
                        const double s0 = sx * sy * sz;
                        const double t0 = b * (2 * (c2.l + c2.m + c2.n) + 3) * s0;
                        const double t1 = -2 * b * b *
                                          (Ex[c1_.l][c2.l + 2][0] * sy * sz + sx * Ey[c1_.m][c2.m + 2][0] * sz +
                                           sx * sy * Ez[c1_.n][c2.n + 2][0]);
                        double t2 = 0.0;
                        if (c2.l >= 2) t2 += c2.l * (c2.l - 1) * Ex[c1_.l][c2.l - 2][0] * sy * sz;
                        if (c2.m >= 2) t2 += c2.m * (c2.m - 1) * sx * Ey[c1_.m][c2.m - 2][0] * sz;
                        if (c2.n >= 2) t2 += c2.n * (c2.n - 1) * sx * sy * Ez[c1_.n][c2.n - 2][0];
                        const double w = pre * ca[i] * cb[j];
                        sacc[i * NB + j] = fma(w, s0, sacc[i * NB + j]);
                        tacc[i * NB + j] = fma(w, t0 + t1 - 0.5 * t2, tacc[i * NB + j]);
                    }
            }
            if (c0 < c1) {
                double Ex[LA + 1][LB + 1][L + 1], Ey[LA + 1][LB + 1][L + 1], Ez[LA + 1][LB + 1][L + 1];
                e1d_ct<LA, LB>(Ex, px - ax, px - bx, 0.5 * ip);
                e1d_ct<LA, LB>(Ey, py - ay, py - by, 0.5 * ip);
                e1d_ct<LA, LB>(Ez, pz - az, pz - bz, 0.5 * ip);
                const double vpre = K * 2 * PI * ip;
                for (int c = c0; c < c1; ++c) {
                    const double X = px - C[3 * c], Y = py - C[3 * c + 1], Zc = pz - C[3 * c + 2];
                    double F[L + 1];
                    boys_scaled<L>(p * (X * X + Y * Y + Zc * Zc), 1.0, -2.0 * p, boys, F);
                    double R[nherm(L)];
                    r_ct<L>(R, F, X, Y, Zc);
                    const double zc = -(double)Z[c] * vpre;
#pragma unroll
                    for (int i = 0; i < NA; ++i)
#pragma unroll
                        for (int j = 0; j < NB; ++j) {
                            const Cart c1_ = cart(LA, i), c2 = cart(LB, j);
                            double acc = 0.0;
#pragma unroll
                            for (int t = 0; t <= c1_.l + c2.l; ++t) {
                                double su = 0.0;
#pragma unroll
                                for (int u = 0; u <= c1_.m + c2.m; ++u) {
                                    double sv = 0.0;
#pragma unroll
                                    for (int v = 0; v <= c1_.n + c2.n; ++v)
                                        sv = fma(Ez[c1_.n][c2.n][v], R[hidx(t, u, v)], sv);
                                    su = fma(Ey[c1_.m][c2.m][u], sv, su);
                                }
                                acc = fma(Ex[c1_.l][c2.l][t], su, acc);
                            }
                            vacc[i * NB + j] = fma(zc * ca[i] * cb[j], acc, vacc[i * NB + j]);
                        }
                }
            }
        }
    const int* fa = sh.comp_fn + sh.cfn0[A];
    const int* fb = sh.comp_fn + sh.cfn0[B];
#pragma unroll
    for (int i = 0; i < NA; ++i)
#pragma unroll
        for (int j = 0; j < NB; ++j) {
            const int x = fa[i], y = fb[j];
            if (x < 0 || y < 0) continue;
            if (A == B && i < j) continue;
            const int64_t o1 = x + (int64_t)y * n, o2 = y + (int64_t)x * n;
            if (st_chunk) {
                if (S) S[o1] = S[o2] = sacc[i * NB + j];
                if (T) T[o1] = T[o2] = tacc[i * NB + j];
            }
            if (V && c0 < c1) {
                atomicAdd(V + o1, vacc[i * NB + j]);
                if (o2 != o1) atomicAdd(V + o2, vacc[i * NB + j]);
            }
        }
}

void onee_compute(Context& ctx, const Basis& b, int nat, const int* atno, const double* x, const double* y,
                  const double* z, double* dS, double* dT, double* dV, cudaStream_t on)
{
    cudaStream_t st = on ? on : ctx.stream;
    const int n = b.nbf;
    const int ns = (int)b.shells.size();
    std::vector<int> L(ns), np(ns), p0(ns), c0(ns), f0(ns);
    std::vector<double> xyz(3 * ns);
    for (int s = 0; s < ns; ++s) {
        const Shell& sh = b.shells[s];
        HF_CHECK(sh.L <= 2, HFGPU_ERR_UNSUPPORTED, "one-electron integrals support s, p and d shells");
        L[s] = sh.L; np[s] = sh.nprim; p0[s] = sh.prim0; c0[s] = sh.coef0; f0[s] = sh.cfn0;
        xyz[3 * s] = sh.x; xyz[3 * s + 1] = sh.y; xyz[3 * s + 2] = sh.z;
    }
    // shell pairs by pair type, the larger angular momentum first
    std::vector<int2> pairs;
    int off[NPTYPE + 1] = {};
    {
        std::vector<std::vector<int2>> by(NPTYPE);
        for (int s1 = 0; s1 < ns; ++s1)
            for (int s2 = 0; s2 <= s1; ++s2) {
                const int A = L[s1] >= L[s2] ? s1 : s2, B = A == s1 ? s2 : s1;
                by[ptype_of(L[A], L[B])].push_back(make_int2(A, B));
            }
        for (int t = 0; t < NPTYPE; ++t) {
            off[t] = (int)pairs.size();
            pairs.insert(pairs.end(), by[t].begin(), by[t].end());
        }
        off[NPTYPE] = (int)pairs.size();
    }
    std::vector<int> Z(nat > 0 ? nat : 1);
    std::vector<double> C(3 * (nat > 0 ? nat : 1));
    for (int i = 0; i < nat; i++) {
        Z[i] = atno[i];
        C[3 * i] = x[i]; C[3 * i + 1] = y[i]; C[3 * i + 2] = z[i];
    }
    auto dL = to_device(L, st);
    auto dn = to_device(np, st);
    auto dp0 = to_device(p0, st);
    auto dc0 = to_device(c0, st);
    auto df0 = to_device(f0, st);
    auto dxyz = to_device(xyz, st);
    auto dal = to_device(b.alpha, st);
    auto dco = to_device(b.coef, st);
    auto dcf = to_device(b.comp_fn, st);
    auto dpairs = to_device(pairs, st);
    auto dZ = to_device(Z, st);
    auto dC = to_device(C, st);
    ShellOne sh{dL.p, dn.p, dp0.p, dc0.p, df0.p, dxyz.p, dal.p, dco.p, dcf.p};
    if (dV) HF_CUDA(cudaMemsetAsync(dV, 0, sizeof(double) * n * n, st));
    const unsigned chunks = (unsigned)std::max(1, (nat + ONEE_ATOMS - 1) / ONEE_ATOMS);
    for (int t = 0; t < NPTYPE; ++t) {
        const int np_t = off[t + 1] - off[t];
        if (np_t == 0) continue;
        const dim3 grid((unsigned)((np_t + 63) / 64), dV ? chunks : 1u);
        const int2* pp = dpairs.p + off[t];
        switch (t) {
            case 0: onee_shell_kernel<0, 0><<<grid, 64, 0, st>>>(sh, pp, np_t, n, nat, dZ.p, dC.p, ctx.boys, dS, dT, dV); break;
            case 1: onee_shell_kernel<1, 0><<<grid, 64, 0, st>>>(sh, pp, np_t, n, nat, dZ.p, dC.p, ctx.boys, dS, dT, dV); break;
            case 2: onee_shell_kernel<2, 0><<<grid, 64, 0, st>>>(sh, pp, np_t, n, nat, dZ.p, dC.p, ctx.boys, dS, dT, dV); break;
            case 3: onee_shell_kernel<1, 1><<<grid, 64, 0, st>>>(sh, pp, np_t, n, nat, dZ.p, dC.p, ctx.boys, dS, dT, dV); break;
            case 4: onee_shell_kernel<2, 1><<<grid, 64, 0, st>>>(sh, pp, np_t, n, nat, dZ.p, dC.p, ctx.boys, dS, dT, dV); break;
            default: onee_shell_kernel<2, 2><<<grid, 64, 0, st>>>(sh, pp, np_t, n, nat, dZ.p, dC.p, ctx.boys, dS, dT, dV); break;
        }
        count_launch();
        HF_CUDA(cudaGetLastError());
    }
}

}  // namespace hfgpu
