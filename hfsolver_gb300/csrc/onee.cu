// One-electron integrals S, T, V over contracted Cartesian GTOs on the GPU.
//
// Same matrices as hfsolver's getS/getT/getV (src/qc.c:6-93 over
// src/cints.c:186-307), evaluated with McMurchie-Davidson expansions:
//   S_ab = sum c_a c_b K_ab (pi/p)^{3/2} Ex^{ab}_0 Ey^{ab}_0 Ez^{ab}_0
//   T_ab from overlaps with the ket power raised/lowered by 2 (the same
//        kinetic formula as cints.c:186-210)
//   V_ab = -sum_C Z_C sum c_a c_b K_ab (2 pi/p) sum_tuv E^{ab}_{tuv} R_tuv(p, P-C)
// One thread per matrix element (i, j) and chunk of nuclei; n x n column-major like
// the reference.
#include <algorithm>
#include <vector>

#include "boys.cuh"
#include "internal.h"
#include "md.cuh"

namespace hfgpu {

struct FnDev {
    const int* lmn;      // 3 per function
    const int* nprim;
    const int* a0;       // offset of the exponents
    const int* c0;       // offset of this component's coefficients
    const double* xyz;   // 3 per function
    const double* alpha;
    const double* coef;
};

constexpr int OE_LA = 2, OE_LB = 4, OE_T = OE_LA + OE_LB + 1;

__device__ static void e1d(double (&E)[OE_LA + 1][OE_LB + 1][OE_T], int la, int lb, double xpa, double xpb,
                           double i2p)
{
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j)
            for (int t = 0; t < OE_T; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
    for (int i = 0; i < la; ++i)
        for (int t = 0; t <= i + 1; ++t) {
            double v = xpa * E[i][0][t];
            if (t > 0) v = fma(i2p, E[i][0][t - 1], v);
            if (t + 1 <= i) v = fma((double)(t + 1), E[i][0][t + 1], v);
            E[i + 1][0][t] = v;
        }
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j < lb; ++j)
            for (int t = 0; t <= i + j + 1; ++t) {
                double v = xpb * E[i][j][t];
                if (t > 0) v = fma(i2p, E[i][j][t - 1], v);
                if (t + 1 <= i + j) v = fma((double)(t + 1), E[i][j][t + 1], v);
                E[i][j + 1][t] = v;
            }
}

constexpr int OE_L = 4;  // largest l_a + l_b for s, p, d

// R_tuv(p, PC) for t+u+v <= L <= OE_L (Helgaker et al. eqs. 9.9.18-9.9.20)
__device__ static void r_aux(int L, double (&R)[OE_L + 1][nherm(OE_L)], const double (&F)[OE_L + 1], double X, double Y,
                             double Z)
{
    for (int n = 0; n <= L; ++n) R[n][0] = F[n];
    for (int n = L - 1; n >= 0; --n)
        for (int s = 1; s <= L - n; ++s)
            for (int t = s; t >= 0; --t)
                for (int v = 0; v <= s - t; ++v) {
                    int u = s - t - v;
                    double r;
                    if (t > 0) {
                        r = X * R[n + 1][hidx(t - 1, u, v)];
                        if (t > 1) r = fma((double)(t - 1), R[n + 1][hidx(t - 2, u, v)], r);
                    } else if (u > 0) {
                        r = Y * R[n + 1][hidx(0, u - 1, v)];
                        if (u > 1) r = fma((double)(u - 1), R[n + 1][hidx(0, u - 2, v)], r);
                    } else {
                        r = Z * R[n + 1][hidx(0, 0, v - 1)];
                        if (v > 1) r = fma((double)(v - 1), R[n + 1][hidx(0, 0, v - 2)], r);
                    }
                    R[n][hidx(t, u, v)] = r;
                }
}

// blockIdx.y = a chunk of ONEE_ATOMS nuclei: chunk 0 also writes S and T; every
// chunk adds its nuclei's attraction to V (zeroed by the caller) atomically.
constexpr int ONEE_ATOMS = 4;

__global__ void onee_kernel(FnDev f, int n, int nat, const int* __restrict__ Z, const double* __restrict__ C,
                            const double* __restrict__ boys, double* S, double* T, double* V)
{
    const double PI = 3.14159265358979323846;
    // one thread per lower-triangle element (i >= j), mirrored on output
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * (n + 1) / 2) return;
    int i = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
    while ((int64_t)i * (i + 1) / 2 > idx) --i;
    while ((int64_t)(i + 1) * (i + 2) / 2 <= idx) ++i;
    const int j = (int)(idx - (int64_t)i * (i + 1) / 2);
    int l1 = f.lmn[3 * i], m1 = f.lmn[3 * i + 1], n1 = f.lmn[3 * i + 2];
    int l2 = f.lmn[3 * j], m2 = f.lmn[3 * j + 1], n2 = f.lmn[3 * j + 2];
    double ax = f.xyz[3 * i], ay = f.xyz[3 * i + 1], az = f.xyz[3 * i + 2];
    double bx = f.xyz[3 * j], by = f.xyz[3 * j + 1], bz = f.xyz[3 * j + 2];
    double rab2 = (ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz);
    double s_acc = 0, t_acc = 0, v_acc = 0;
    for (int pa = 0; pa < f.nprim[i]; ++pa)
        for (int pb = 0; pb < f.nprim[j]; ++pb) {
            double a = f.alpha[f.a0[i] + pa], b = f.alpha[f.a0[j] + pb];
            double cc = f.coef[f.c0[i] + pa] * f.coef[f.c0[j] + pb];
            double p = a + b, ip = 1.0 / p;
            double px = (a * ax + b * bx) * ip, py = (a * ay + b * by) * ip, pz = (a * az + b * bz) * ip;
            double K = exp(-a * b * ip * rab2);
            double Ex[OE_LA + 1][OE_LB + 1][OE_T], Ey[OE_LA + 1][OE_LB + 1][OE_T], Ez[OE_LA + 1][OE_LB + 1][OE_T];
            e1d(Ex, l1, l2 + 2, px - ax, px - bx, 0.5 * ip);
            e1d(Ey, m1, m2 + 2, py - ay, py - by, 0.5 * ip);
            e1d(Ez, n1, n2 + 2, pz - az, pz - bz, 0.5 * ip);
            double pre = cc * K * PI * ip * sqrt(PI * ip);
            // overlap and kinetic (cints.c:186-232 in terms of 1-D overlaps)
            double sx = Ex[l1][l2][0], sy = Ey[m1][m2][0], sz = Ez[n1][n2][0];
            double s0 = sx * sy * sz;
            double t0 = b * (2 * (l2 + m2 + n2) + 3) * s0;
            double t1 = -2 * b * b *
                        (Ex[l1][l2 + 2][0] * sy * sz + sx * Ey[m1][m2 + 2][0] * sz + sx * sy * Ez[n1][n2 + 2][0]);
            double t2 = 0;
            if (l2 >= 2) t2 += l2 * (l2 - 1) * Ex[l1][l2 - 2][0] * sy * sz;
            if (m2 >= 2) t2 += m2 * (m2 - 1) * sx * Ey[m1][m2 - 2][0] * sz;
            if (n2 >= 2) t2 += n2 * (n2 - 1) * sx * sy * Ez[n1][n2 - 2][0];
            s_acc += pre * s0;
            t_acc += pre * (t0 + t1 - 0.5 * t2);
            // nuclear attraction of this block's nuclei
            double vsum = 0;
            const int c0 = blockIdx.y * ONEE_ATOMS, c1 = min(nat, c0 + ONEE_ATOMS);
            for (int c = c0; c < c1; ++c) {
                double X = px - C[3 * c], Y = py - C[3 * c + 1], Zc = pz - C[3 * c + 2];
                double F[OE_L + 1];
                const double Tc = p * (X * X + Y * Y + Zc * Zc);
                const int L = l1 + l2 + m1 + m2 + n1 + n2;
                switch (L) {  // Boys values up to the order this pair needs
                    case 0: { double f[1]; boys_scaled<0>(Tc, 1.0, -2.0 * p, boys, f); F[0] = f[0]; break; }
                    case 1: { double f[2]; boys_scaled<1>(Tc, 1.0, -2.0 * p, boys, f); for (int k = 0; k < 2; ++k) F[k] = f[k]; break; }
                    case 2: { double f[3]; boys_scaled<2>(Tc, 1.0, -2.0 * p, boys, f); for (int k = 0; k < 3; ++k) F[k] = f[k]; break; }
                    case 3: { double f[4]; boys_scaled<3>(Tc, 1.0, -2.0 * p, boys, f); for (int k = 0; k < 4; ++k) F[k] = f[k]; break; }
                    default: boys_scaled<OE_L>(Tc, 1.0, -2.0 * p, boys, F); break;
                }
                double R[OE_L + 1][nherm(OE_L)];
                r_aux(L, R, F, X, Y, Zc);
                double acc = 0;
                for (int t = 0; t <= l1 + l2; ++t)
                    for (int u = 0; u <= m1 + m2; ++u)
                        for (int v = 0; v <= n1 + n2; ++v)
                            acc += Ex[l1][l2][t] * Ey[m1][m2][u] * Ez[n1][n2][v] * R[0][hidx(t, u, v)];
                vsum -= Z[c] * acc;
            }
            v_acc += cc * K * 2 * PI * ip * vsum;
        }
    const int64_t o1 = i + (int64_t)j * n, o2 = j + (int64_t)i * n;
    if (blockIdx.y == 0) {
        if (S) S[o1] = S[o2] = s_acc;
        if (T) T[o1] = T[o2] = t_acc;
    }
    if (V && v_acc != 0.0) {
        atomicAdd(V + o1, v_acc);
        if (o2 != o1) atomicAdd(V + o2, v_acc);
    }
}

void onee_compute(Context& ctx, const Basis& b, int nat, const int* atno, const double* x, const double* y,
                  const double* z, double* dS, double* dT, double* dV, cudaStream_t on)
{
    cudaStream_t st = on ? on : ctx.stream;
    int n = b.nbf;
    std::vector<int> lmn(3 * n), np(n), a0(n), c0(n);
    std::vector<double> xyz(3 * n);
    for (auto& sh : b.shells)
        for (int c = 0; c < ncart(sh.L); c++) {
            int fn = b.comp_fn[sh.cfn0 + c];
            if (fn < 0) continue;
            Cart cc = cart(sh.L, c);
            lmn[3 * fn] = cc.l; lmn[3 * fn + 1] = cc.m; lmn[3 * fn + 2] = cc.n;
            np[fn] = sh.nprim;
            a0[fn] = sh.prim0;
            c0[fn] = sh.coef0 + c * sh.nprim;
            xyz[3 * fn] = sh.x; xyz[3 * fn + 1] = sh.y; xyz[3 * fn + 2] = sh.z;
        }
    std::vector<int> Z(nat > 0 ? nat : 1);
    std::vector<double> C(3 * (nat > 0 ? nat : 1));
    for (int i = 0; i < nat; i++) {
        Z[i] = atno[i];
        C[3 * i] = x[i]; C[3 * i + 1] = y[i]; C[3 * i + 2] = z[i];
    }
    auto dl = to_device(lmn, st);
    auto dn = to_device(np, st);
    auto da = to_device(a0, st);
    auto dc = to_device(c0, st);
    auto dx = to_device(xyz, st);
    auto dal = to_device(b.alpha, st);
    auto dco = to_device(b.coef, st);
    auto dZ = to_device(Z, st);
    auto dC = to_device(C, st);
    FnDev f{dl.p, dn.p, da.p, dc.p, dx.p, dal.p, dco.p};
    const int64_t npair = (int64_t)n * (n + 1) / 2;
    if (dV) HF_CUDA(cudaMemsetAsync(dV, 0, sizeof(double) * n * n, st));
    const dim3 grid((unsigned)((npair + 127) / 128), (unsigned)std::max(1, (nat + ONEE_ATOMS - 1) / ONEE_ATOMS));
    onee_kernel<<<grid, 128, 0, st>>>(f, n, nat, dZ.p, dC.p, ctx.boys, dS, dT, dV);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

}  // namespace hfgpu
