// Analytic RHF nuclear gradient on sm_103a.
//
// hfsolver has no gradient code.  This is the derivative, with respect to the
// nuclear positions, of the energy that doscf minimises (src/scf.f90:72-150),
// for the force callback of src/md.f90:13-20:
//   dE/dX = sum_ab P_ab dH_ab/dX - sum_ab W_ab dS_ab/dX
//         + sum_abcd Gamma_abcd d(ab|cd)/dX + dE_nuc/dX
//   P = 2 C_occ C_occ^T,  W = 2 C_occ diag(eps_occ) C_occ^T,
//   Gamma_abcd = P_ab P_cd / 2 - (P_ac P_bd + P_ad P_bc) / 8.
// A Cartesian Gaussian's derivative with respect to its centre raises and
// lowers its power:
//   d/dAx [x_A^i exp(-a x_A^2)] = 2a x_A^{i+1} exp(-a x_A^2) - i x_A^{i-1} exp(-a x_A^2),
// so every derivative integral is a sum of integrals whose McMurchie-Davidson
// coefficients come from 1-D tables with one more unit of angular momentum.
//
// Two-electron part (adjoint form): derivative integrals are never stored.
// Per ordered quartet class, generated kernels (gen_grad.py, grad_kernel.cuh)
// differentiate one pair of each screened quartet: the other pair's
// primitives are summed first into Hermite intermediates
//   X_cd(tau) = sum_{ket prims} sum_tau' (-1)^{|tau'|} E^{cd}_tau' R_{tau+tau'}
// (R up to order L+1), which are then contracted once per bra primitive pair
// with Gamma8 = 8 Gamma and the bra's derivative coefficients:
//   g_A += sum_ab Gamma8 c_a c_b sum_tau (d_A E^{ab})_tau X_cd(tau),
//   g_A + g_B from the Hermite shift tau -> tau + 1 (both centres moved).
// A second launch with the pairs swapped gives g_C, and g_D follows from
// translational invariance.  The quartets are those the energy path evaluated
// (same Schwarz screening).
//
// One-electron part: one thread per basis-function pair and pair of nuclei; dS/dA and dT/dA from
// shifted 1-D overlaps (dB = -dA for two-centre integrals), dV from the shifted
// Hermite sums with the Hellmann-Feynman term of each nucleus C obtained by
// translational invariance, dV/dC = -(dV/dA + dV/dB).
#include <algorithm>
#include <mutex>
#include <cmath>
#include <vector>

#include "boys.cuh"
#include "eri_plan.h"
#include "grad_kernel.cuh"
#include "internal.h"
#include "md.cuh"

namespace hfgpu {
// ------------------------------------------------------------- 1-D tables
// E[i][j][t] for i <= la+1, j <= lb+1, t <= i+j, zero elsewhere
constexpr int GE_I = 4, GE_J = 4, GE_T = 7;
constexpr int GE_DIM = GE_I * GE_J * GE_T;

__device__ __forceinline__ int ge(int i, int j, int t) { return (i * GE_J + j) * GE_T + t; }

// runtime-order Hermite expansion coefficients (Helgaker et al. eqs. 9.5.6-9.5.7)
__device__ static void e1d_rt(double* E, int imax, int jmax, double xpa, double xpb, double i2p)
{
    for (int k = 0; k < GE_DIM; ++k) E[k] = 0.0;
    E[ge(0, 0, 0)] = 1.0;
    for (int i = 0; i < imax; ++i)
        for (int t = 0; t <= i + 1; ++t) {
            double v = xpa * E[ge(i, 0, t)];
            if (t > 0) v = fma(i2p, E[ge(i, 0, t - 1)], v);
            if (t + 1 <= i) v = fma((double)(t + 1), E[ge(i, 0, t + 1)], v);
            E[ge(i + 1, 0, t)] = v;
        }
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j < jmax; ++j)
            for (int t = 0; t <= i + j + 1; ++t) {
                double v = xpb * E[ge(i, j, t)];
                if (t > 0) v = fma(i2p, E[ge(i, j, t - 1)], v);
                if (t + 1 <= i + j) v = fma((double)(t + 1), E[ge(i, j, t + 1)], v);
                E[ge(i, j + 1, t)] = v;
            }
}

// one thread per primitive pair of every shell pair
// one thread per primitive pair of every shell pair: the bra-side record of
// the gradient kernels (layout in grad_kernel.cuh: header, then the 1-D
// Hermite coefficients E and the derivative coefficients
// D(i, j, t) = 2a E(i+1, j, t) - i E(i-1, j, t) of each axis)
__global__ void grad_pair_kernel(const int* __restrict__ sL, const int* __restrict__ snp, const int* __restrict__ sp0,
                                 const int* __restrict__ sc0, const double* __restrict__ sxyz,
                                 const double* __restrict__ alpha, const double* __restrict__ coef,
                                 const int* __restrict__ pA, const int* __restrict__ pB, const int2* __restrict__ items,
                                 int nitems, const int64_t* __restrict__ goff, double* __restrict__ gd)
{
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nitems) return;
    const int2 item = items[it];  // (pair, primitive pair within the pair)
    const int P = item.x;
    const int A = pA[P], B = pB[P];
    const int la = sL[A], lb = sL[B];
    const int npa = snp[A], nb = snp[B];
    const int ia = item.y / nb, ib = item.y - ia * nb;  // ia-major, as in the energy records
    double* rec = gd + goff[P] + (int64_t)item.y * grad_stride(la, lb);
    const double a = alpha[sp0[A] + ia], b = alpha[sp0[B] + ib];
    const double ax = sxyz[3 * A], ay = sxyz[3 * A + 1], az = sxyz[3 * A + 2];
    const double bx = sxyz[3 * B], by = sxyz[3 * B + 1], bz = sxyz[3 * B + 2];
    const double p = a + b, ip = 1.0 / p, mu = a * b * ip;
    const double px = (a * ax + b * bx) * ip, py = (a * ay + b * by) * ip, pz = (a * az + b * bz) * ip;
    const double rab2 = (ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz);
    const double kab = exp(-mu * rab2) * ip;
    rec[0] = a;
    rec[1] = b;
    rec[2] = p;
    rec[3] = px;
    rec[4] = py;
    rec[5] = pz;
    rec[6] = kab;
    rec[7] = 0.0;
    for (int c = 0; c < 6; ++c) {
        rec[8 + c] = c < ncart(la) ? coef[sc0[A] + c * npa + ia] * kab : 0.0;
        rec[14 + c] = c < ncart(lb) ? coef[sc0[B] + c * nb + ib] : 0.0;
    }
    const int ts = grad_table(la, lb), tw = la + lb + 2;
    const double xa[3] = {px - ax, py - ay, pz - az}, xb[3] = {px - bx, py - by, pz - bz};
    double E[GE_DIM];
    for (int d = 0; d < 3; ++d) {
        e1d_rt(E, la + 1, lb, xa[d], xb[d], 0.5 * ip);
        double* te = rec + GR_HDR + d * ts;
        double* td = rec + GR_HDR + (3 + d) * ts;
        for (int i = 0; i <= la; ++i)
            for (int j = 0; j <= lb; ++j)
                for (int t = 0; t < tw; ++t) {
                    const int o = (i * (lb + 1) + j) * tw + t;
                    te[o] = t <= i + j ? E[ge(i, j, t)] : 0.0;
                    const double up = E[ge(i + 1, j, t)];
                    const double dn = (i > 0 && t <= i + j - 1) ? E[ge(i - 1, j, t)] : 0.0;
                    td[o] = 2.0 * a * up - (double)i * dn;
                }
    }
}

__device__ static void boys_rt(int M, double T, double pref, double s, const double* __restrict__ tab, double* F)
{
    if (T < BOYS_TMAX) {
        const int k = __double2int_rn(T * 16.0);
        const double d = (double)k * BOYS_H - T;
        const double* row = tab + k * BOYS_STRIDE;
        double w[BOYS_NTAYLOR];
        w[0] = 1.0;
#pragma unroll
        for (int j = 1; j < BOYS_NTAYLOR; ++j) w[j] = w[j - 1] * d * (1.0 / j);
        double fm = 0.0, ex = 0.0;
#pragma unroll
        for (int j = BOYS_NTAYLOR - 1; j >= 0; --j) {
            fm = fma(__ldg(row + M + j), w[j], fm);
            ex += w[j];
        }
        const double e = ex * __ldg(row + BOYS_NCOL);
        F[M] = fm;
        for (int m = M - 1; m >= 0; --m) F[m] = fma(2.0 * T, F[m + 1], e) / (double)(2 * m + 1);
    } else {
        const double r = rsqrt_nr(T);
        const double e = (T < 103.0) ? (double)expf(-(float)T) : 0.0;
        const double inv2t = 0.5 * r * r;
        double f = 0.88622692545275801364 * r;
        F[0] = f;
        for (int m = 0; m < M; ++m) {
            f = fma((double)(2 * m + 1), f, -e) * inv2t;
            F[m + 1] = f;
        }
    }
    double sc = pref;
    for (int m = 0; m <= M; ++m) {
        F[m] *= sc;
        sc *= s;
    }
}

// ------------------------------------------------------------- two-electron part
// (the class kernels: grad_kernel.cuh and gen/grad_class_*.cu)

// ------------------------------------------------------------- one-electron part
// Two passes.  onee_grad_pair_kernel: one thread per primitive pair of a shell
// pair adds the overlap and kinetic terms and leaves the nuclear-attraction
// derivatives of all its component pairs folded into six Hermite densities,
//   H_{A,k}(tau) = sum_ab w_ab c_a c_b (2a E^{a+1_k, b}_tau - a_k E^{a-1_k, b}_tau)
//   H_{B,k}(tau) = sum_ab w_ab c_a c_b (2b E^{a, b+1_k}_tau - b_k E^{a, b-1_k}_tau)
// (w = the density P counted for both triangle entries, |tau| <= l_A + l_B + 1).
// onee_grad_nuc_kernel: one thread per (primitive pair, nucleus C) evaluates
// R_tuv(p, P - C) once and contracts it with the six densities:
//   dV/dA_k = -Z_C K 2pi/p sum_tau H_{A,k}(tau) R_tau (and B), and the
// Hellmann-Feynman term of C is -(dV/dA + dV/dB).
struct OnePairArgs {
    const int* sL;
    const int* snp;
    const int* sp0;
    const int* sc0;
    const int* scf;
    const int* satom;
    const double* sxyz;
    const double* alpha;
    const double* coef;
    const int* comp_fn;
    const double* P;
    const double* W;
    int n, nat;
    const int4* items;  // (shell A, shell B, primitive pair, record offset in doubles)
    int nitems;
    double* rec;        // per primitive pair: header (8) + 6 densities of nherm(l_A + l_B + 1)
    double* grad;
};

constexpr int OG_HDR = 8;  // p, Px, Py, Pz, K 2pi/p, atom A, atom B, unused

constexpr int OG_I = 4, OG_J = 6, OG_T = 9;  // i <= la+1, j <= lb+3, t <= i+j (only t <= 5 used)
constexpr int OG_L = 5;                     // la + lb + 1
__device__ __forceinline__ int og(int i, int j, int t) { return (i * OG_J + j) * OG_T + t; }

__device__ static void e1d_oe(double* E, int imax, int jmax, double xpa, double xpb, double i2p)
{
    for (int k = 0; k < OG_I * OG_J * OG_T; ++k) E[k] = 0.0;
    E[og(0, 0, 0)] = 1.0;
    for (int i = 0; i < imax; ++i)
        for (int t = 0; t <= i + 1 && t < OG_T; ++t) {
            double v = xpa * E[og(i, 0, t)];
            if (t > 0) v = fma(i2p, E[og(i, 0, t - 1)], v);
            if (t + 1 <= i) v = fma((double)(t + 1), E[og(i, 0, t + 1)], v);
            E[og(i + 1, 0, t)] = v;
        }
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j < jmax; ++j)
            for (int t = 0; t <= i + j + 1 && t < OG_T; ++t) {
                double v = xpb * E[og(i, j, t)];
                if (t > 0) v = fma(i2p, E[og(i, j, t - 1)], v);
                if (t + 1 <= i + j && t + 1 < OG_T) v = fma((double)(t + 1), E[og(i, j, t + 1)], v);
                E[og(i, j + 1, t)] = v;
            }
}

__global__ void onee_grad_pair_kernel(OnePairArgs o)
{
    const double PI = 3.14159265358979323846;
    extern __shared__ double sg[];  // 3 per nucleus
    for (int k = threadIdx.x; k < 3 * o.nat; k += blockDim.x) sg[k] = 0.0;
    __syncthreads();
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it < o.nitems) {
        const int4 item = o.items[it];
        const int A = item.x, B = item.y;
        const int la = o.sL[A], lb = o.sL[B];
        const int npa = o.snp[A], npb = o.snp[B];
        const int pa = item.z / npb, pb = item.z - pa * npb;
        const double a = o.alpha[o.sp0[A] + pa], b = o.alpha[o.sp0[B] + pb];
        const double Ax[3] = {o.sxyz[3 * A], o.sxyz[3 * A + 1], o.sxyz[3 * A + 2]};
        const double Bx[3] = {o.sxyz[3 * B], o.sxyz[3 * B + 1], o.sxyz[3 * B + 2]};
        const double p = a + b, ip = 1.0 / p;
        double Pc[3], rab2 = 0.0;
        double E[3][OG_I * OG_J * OG_T];
        for (int k = 0; k < 3; ++k) {
            Pc[k] = (a * Ax[k] + b * Bx[k]) * ip;
            rab2 += (Ax[k] - Bx[k]) * (Ax[k] - Bx[k]);
            e1d_oe(E[k], la + 1, lb + 3, Pc[k] - Ax[k], Pc[k] - Bx[k], 0.5 * ip);
        }
        const double K = exp(-a * b * ip * rab2);
        const double pre = K * PI * ip * sqrt(PI * ip);
        const int L = la + lb + 1, nh = nherm(L);
        double* h = o.rec + item.w;
        h[0] = p;
        h[1] = Pc[0];
        h[2] = Pc[1];
        h[3] = Pc[2];
        h[4] = K * 2 * PI * ip;
        h[5] = (double)o.satom[A];
        h[6] = (double)o.satom[B];
        h[7] = 0.0;
        double* H = h + OG_HDR;
        for (int k = 0; k < 6 * nh; ++k) H[k] = 0.0;
        const int* fa = o.comp_fn + o.scf[A];
        const int* fb = o.comp_fn + o.scf[B];
        const double* coA = o.coef + o.sc0[A];
        const double* coB = o.coef + o.sc0[B];
        auto s1 = [&](int k, int ii, int jj) -> double { return (ii < 0 || jj < 0) ? 0.0 : E[k][og(ii, jj, 0)]; };
        double gA[3] = {0, 0, 0};
        for (int i = 0; i < ncart(la); ++i)
            for (int j = 0; j < ncart(lb); ++j) {
                if (A == B && i < j) continue;
                const int x = fa[i], y = fb[j];
                if (x < 0 || y < 0) continue;
                const double sym = (A == B && i == j) ? 1.0 : 2.0;
                const double cc = coA[i * npa + pa] * coB[j * npb + pb];
                const double wP = sym * o.P[x + (int64_t)y * o.n], wW = sym * o.W[x + (int64_t)y * o.n];
                const Cart ca = cart(la, i), cb = cart(lb, j);
                const int qa[3] = {ca.l, ca.m, ca.n}, qb[3] = {cb.l, cb.m, cb.n};
                // overlap and kinetic (cints.c:186-232 in terms of 1-D overlaps)
                auto st = [&](const int* q, double& sv, double& tv) {
                    const double sx = s1(0, q[0], qb[0]), sy = s1(1, q[1], qb[1]), sz = s1(2, q[2], qb[2]);
                    sv = sx * sy * sz;
                    const double t0 = b * (2 * (qb[0] + qb[1] + qb[2]) + 3) * sv;
                    const double t1 = -2 * b * b *
                                      (s1(0, q[0], qb[0] + 2) * sy * sz + sx * s1(1, q[1], qb[1] + 2) * sz +
                                       sx * sy * s1(2, q[2], qb[2] + 2));
                    const double t2 = qb[0] * (qb[0] - 1) * s1(0, q[0], qb[0] - 2) * sy * sz +
                                      qb[1] * (qb[1] - 1) * sx * s1(1, q[1], qb[1] - 2) * sz +
                                      qb[2] * (qb[2] - 1) * sx * sy * s1(2, q[2], qb[2] - 2);
                    tv = t0 + t1 - 0.5 * t2;
                };
                for (int k = 0; k < 3; ++k) {
                    int up[3] = {qa[0], qa[1], qa[2]}, dn[3] = {qa[0], qa[1], qa[2]};
                    up[k] += 1;
                    dn[k] -= 1;
                    double su, tu, sd = 0, td = 0;
                    st(up, su, tu);
                    if (qa[k] > 0) st(dn, sd, td);
                    const double dS = pre * cc * (2 * a * su - qa[k] * sd);
                    const double dT = pre * cc * (2 * a * tu - qa[k] * td);
                    gA[k] += wP * dT - wW * dS;  // two-centre: d/dB = -d/dA
                }
                // nuclear attraction: the six Hermite densities, over each derivative's
                // support only (the component pair's box, one longer along k)
                const double w = wP * cc;
                for (int k = 0; k < 3; ++k) {
                    const int tmax[3] = {qa[0] + qb[0] + (k == 0), qa[1] + qb[1] + (k == 1), qa[2] + qb[2] + (k == 2)};
                    for (int t = 0; t <= tmax[0]; ++t)
                        for (int u = 0; u <= tmax[1]; ++u)
                            for (int v = 0; v <= tmax[2]; ++v) {
                                const int tt[3] = {t, u, v};
                                double eA = w, eB = w;
                                for (int d = 0; d < 3; ++d) {
                                    if (d == k) {
                                        const double up = E[d][og(qa[d] + 1, qb[d], tt[d])];
                                        const double dn = qa[d] > 0 ? E[d][og(qa[d] - 1, qb[d], tt[d])] : 0.0;
                                        eA *= 2 * a * up - qa[d] * dn;
                                        const double ub = E[d][og(qa[d], qb[d] + 1, tt[d])];
                                        const double db = qb[d] > 0 ? E[d][og(qa[d], qb[d] - 1, tt[d])] : 0.0;
                                        eB *= 2 * b * ub - qb[d] * db;
                                    } else {
                                        const double e = E[d][og(qa[d], qb[d], tt[d])];
                                        eA *= e;
                                        eB *= e;
                                    }
                                }
                                const int hh = hidx(t, u, v);
                                H[k * nh + hh] += eA;
                                H[(3 + k) * nh + hh] += eB;
                            }
                }
            }
        const int ta = 3 * o.satom[A], tb = 3 * o.satom[B];
        for (int k = 0; k < 3; ++k) {
            if (gA[k] != 0.0) {
                atomicAdd(sg + ta + k, gA[k]);
                atomicAdd(sg + tb + k, -gA[k]);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * o.nat; k += blockDim.x)
        if (sg[k] != 0.0) atomicAdd(o.grad + k, sg[k]);
}

template <int L>
__global__ void __launch_bounds__(128) onee_grad_nuc_kernel(const double* __restrict__ rec, int nrec, int nat,
                                                            const int* __restrict__ Z, const double* __restrict__ C,
                                                            const double* __restrict__ boys, double* grad)
{
    constexpr int NH = nherm(L);
    extern __shared__ double sg[];  // 3 per nucleus
    for (int k = threadIdx.x; k < 3 * nat; k += blockDim.x) sg[k] = 0.0;
    __syncthreads();
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < (int64_t)nrec * nat) {
        const int r = (int)(idx / nat), c = (int)(idx - (int64_t)r * nat);
        const double* h = rec + (int64_t)r * (OG_HDR + 6 * NH);
        const double p = __ldg(h);
        const double X = __ldg(h + 1) - C[3 * c], Y = __ldg(h + 2) - C[3 * c + 1], Zc = __ldg(h + 3) - C[3 * c + 2];
        double F[L + 1];
        boys_scaled<L>(p * (X * X + Y * Y + Zc * Zc), 1.0, -2.0 * p, boys, F);
        double R[NH];
        r_ct<L>(R, F, X, Y, Zc);
        const double zc = -(double)Z[c] * __ldg(h + 4);
        const int ta = 3 * (int)__ldg(h + 5), tb = 3 * (int)__ldg(h + 6);
        const double* H = h + OG_HDR;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double sA = 0.0, sB = 0.0;
#pragma unroll
            for (int t = 0; t < NH; ++t) {
                sA = fma(__ldg(H + k * NH + t), R[t], sA);
                sB = fma(__ldg(H + (3 + k) * NH + t), R[t], sB);
            }
            const double dA = zc * sA, dB = zc * sB;
            atomicAdd(sg + ta + k, dA);
            atomicAdd(sg + tb + k, dB);
            atomicAdd(sg + 3 * c + k, -(dA + dB));
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * nat; k += blockDim.x)
        if (sg[k] != 0.0) atomicAdd(grad + k, sg[k]);
}

// ------------------------------------------------------------- host side
#define HF_GDECL(B, K) GradKernelFn grad_kernel_##B##K(bool withp);
HF_GDECL(0, 0) HF_GDECL(0, 1) HF_GDECL(0, 2) HF_GDECL(0, 3) HF_GDECL(0, 4) HF_GDECL(0, 5)
HF_GDECL(1, 0) HF_GDECL(1, 1) HF_GDECL(1, 2) HF_GDECL(1, 3) HF_GDECL(1, 4) HF_GDECL(1, 5)
HF_GDECL(2, 0) HF_GDECL(2, 1) HF_GDECL(2, 2) HF_GDECL(2, 3) HF_GDECL(2, 4) HF_GDECL(2, 5)
HF_GDECL(3, 0) HF_GDECL(3, 1) HF_GDECL(3, 2) HF_GDECL(3, 3) HF_GDECL(3, 4) HF_GDECL(3, 5)
HF_GDECL(4, 0) HF_GDECL(4, 1) HF_GDECL(4, 2) HF_GDECL(4, 3) HF_GDECL(4, 4) HF_GDECL(4, 5)
HF_GDECL(5, 0) HF_GDECL(5, 1) HF_GDECL(5, 2) HF_GDECL(5, 3) HF_GDECL(5, 4) HF_GDECL(5, 5)
#undef HF_GDECL

static GradKernelFn get_grad_kernel(int tb, int tk, bool withp)
{
#define HF_GROW(B) {grad_kernel_##B##0, grad_kernel_##B##1, grad_kernel_##B##2, grad_kernel_##B##3, grad_kernel_##B##4, grad_kernel_##B##5}
    static GradKernelFn (*const table[6][6])(bool) = {HF_GROW(0), HF_GROW(1), HF_GROW(2), HF_GROW(3), HF_GROW(4), HF_GROW(5)};
#undef HF_GROW
    return table[tb][tk](withp);
}

// lanes per quartet: enough primitive quartets per lane (16 to 32), so that a
// quartet with many primitives does not hold its warp long after the others
static int grad_split(int kb, int kk)
{
    int s = 1;
    while (s < 32 && (int64_t)kb * kk >= 2 * 16 * (int64_t)s) s <<= 1;
    return s;
}

// the max dynamic shared memory of the kernels that have been raised so far
static std::mutex g_smem_mu;

void eri_gradient(Context& ctx, EriPlan* P, const double* dP, double* d_grad, float* ms_out)
{
    cudaStream_t st = ctx.stream;
    const Basis& b = P->basis;
    const int ns = (int)b.shells.size();
    std::vector<int> sat(ns);
    int nat = 0;
    for (int s = 0; s < ns; ++s) {
        HF_CHECK(b.shells[s].atom >= 0, HFGPU_ERR_UNSUPPORTED, "gradient needs a basis built from atoms");
        HF_CHECK(b.shells[s].L <= 2, HFGPU_ERR_UNSUPPORTED, "gradient supports s, p and d shells");
        sat[s] = b.shells[s].atom;
        nat = std::max(nat, sat[s] + 1);
    }
    constexpr int MAX_GAM = 36;  // largest NAB x NCDC of any ordered class (a dd bra)
    const size_t smem_max = ((size_t)MAX_GAM * GRAD_BLK + 3 * (size_t)nat) * sizeof(double);
    HF_CHECK(smem_max <= 200 * 1024, HFGPU_ERR_UNSUPPORTED, "gradient: too many atoms for the per-block sums");
    // gradient pair records: pair P's records are consecutive, (ia, ib) ia-major
    std::vector<int64_t> goff(P->npair);
    std::vector<int2> items;
    int64_t nrec = 0;
    for (int id = 0; id < P->npair; ++id) {
        goff[id] = nrec;
        const int la = b.shells[P->pA[id]].L, lb = b.shells[P->pB[id]].L;
        for (int k = 0; k < P->pK[id]; ++k) items.push_back(make_int2(id, k));
        nrec += (int64_t)P->pK[id] * grad_stride(la, lb);
    }
    DBuf<double> gd((size_t)std::max<int64_t>(nrec, 1), st);
    DBuf<int2> dit = to_device(items, st);
    DBuf<int64_t> dgoff = to_device(goff, st);
    {
        const int ni = (int)items.size();
        if (ni > 0) {
            grad_pair_kernel<<<(ni + 127) / 128, 128, 0, st>>>(P->sL.p, P->snp.p, P->sp0.p, P->sc0.p, P->sxyz.p,
                                                              P->alpha.p, P->coef.p, P->dA.p, P->dB.p, dit.p, ni,
                                                              dgoff.p, gd.p);
            count_launch();
            HF_CUDA(cudaGetLastError());
        }
    }
    DBuf<int> dsat = to_device(sat, st);
    ctx.trace_mark("grad pair data");

    // two launches per class: the bra side of (tb, tk), then its ket side as
    // the swapped class (tk, tb); each with its own warp layout
    struct Launch {
        GradKernelFn fn;
        int64_t nwarps;
        int gam;
        int seg0, nseg;
        double work;  // primitive quartets x component quartets, for the launch order
    };
    std::vector<Launch> launches;
    std::vector<Seg> segs;
    for (int i = (int)P->classes.size() - 1; i >= 0; --i) {
        const ClassPlan& c = P->classes[i];
        if (c.nq == 0) continue;
        for (int side = 0; side < 2; ++side) {
            const int tb = side == 0 ? c.tb : c.tk, tk = side == 0 ? c.tk : c.tb;
            const int G = ncart(ptype_la(tk)) * ncart(ptype_lb(tk)) / grad_ncd(tb, tk);
            Launch l;
            l.fn = get_grad_kernel(tb, tk, side == 0);
            HF_CHECK(l.fn != nullptr, HFGPU_ERR_UNSUPPORTED, "missing gradient kernel");
            l.gam = ncart(ptype_la(tb)) * ncart(ptype_lb(tb)) * grad_ncd(tb, tk);
            l.seg0 = (int)segs.size();
            l.nwarps = 0;
            l.work = 0;
            for (const Seg& s0 : c.segs) {
                HF_CHECK(s0.list == 0, HFGPU_ERR_UNSUPPORTED, "gradient expects prefix-mode segments");
                Seg s = s0;
                const int kbra = P->pK[P->h_gpairs[s0.bra0]], kket = P->pK[P->h_gpairs[s0.ket0]];
                s.split = side == 0 ? grad_split(kbra, kket) : grad_split(kket, kbra);
                s.warp0 = l.nwarps;
                const int64_t qpw = 32 / s.split;
                l.nwarps += (s.nq + qpw - 1) / qpw * G;
                l.work += (double)s.nq * kbra * kket * ncart(ptype_la(tb)) * ncart(ptype_lb(tb)) *
                          ncart(ptype_la(tk)) * ncart(ptype_lb(tk));
                segs.push_back(s);
            }
            l.nseg = (int)segs.size() - l.seg0;
            HF_CHECK(l.nwarps < ((int64_t)1 << 31), HFGPU_ERR_UNSUPPORTED, "gradient class too large");
            launches.push_back(l);
        }
    }
    DBuf<Seg> dsegs = to_device(segs, st);
    // the launches are independent (their sums meet in atomics): spread them over
    // the side streams, smallest first, so that the large ones come last and
    // fill the GPU to the end instead of small ones leaving a ragged tail
    std::sort(launches.begin(), launches.end(),
              [](const Launch& x, const Launch& y) { return x.work < y.work; });
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    HF_CUDA(cudaEventRecord(e0, st));
    ctx.fork();
    int slot = 0;
    for (const Launch& l : launches) {
        cudaStream_t ls = ctx.aux[slot++ % Context::NAUX];
        GradArgs a;
        a.pA = P->dA.p; a.pB = P->dB.p; a.pK = P->dK.p;
        a.poff = P->doff.p; a.pdata = P->pdata.p;
        a.goff = dgoff.p; a.gdata = gd.p;
        a.boys = ctx.boys;
        a.gpairs = P->gpairs.p; a.prefix = P->prefix.p;
        a.segs = dsegs.p + l.seg0; a.nseg = l.nseg; a.nwarps = l.nwarps;
        a.cfn0 = P->scf.p; a.comp_fn = P->cfn.p; a.sat = dsat.p;
        a.P = dP; a.n = b.nbf; a.nat = nat;
        a.gam_stride = l.gam;
        a.grad = d_grad;
        const size_t smem = ((size_t)l.gam * GRAD_BLK + 3 * (size_t)nat) * sizeof(double);
        {
            std::lock_guard<std::mutex> lk(g_smem_mu);
            static std::vector<std::pair<GradKernelFn, size_t>> raised;
            bool ok = false;
            for (auto& r : raised)
                if (r.first == l.fn && r.second >= smem) ok = true;
            if (!ok && smem > 48 * 1024) {
                HF_CUDA(cudaFuncSetAttribute(l.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
                raised.push_back({l.fn, smem_max});
            }
        }
        const int64_t blocks = (l.nwarps + GRAD_BLK / 32 - 1) / (GRAD_BLK / 32);
        l.fn<<<(unsigned)blocks, GRAD_BLK, smem, ls>>>(a);
        count_launch();
        HF_CUDA(cudaGetLastError());
    }
    ctx.join();
    HF_CUDA(cudaEventRecord(e1, st));
    HF_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms_out) *ms_out = ms;
}


void onee_gradient(Context& ctx, const Basis& b, int nat, const int* atno, const double* xyz, const double* dP,
                   const double* dW, double* d_grad)
{
    cudaStream_t st = ctx.stream;
    const int n = b.nbf;
    const int ns = (int)b.shells.size();
    std::vector<int> sL(ns), snp(ns), sp0(ns), sc0(ns), scf(ns), sat(ns);
    std::vector<double> sxyz(3 * ns);
    for (int s = 0; s < ns; ++s) {
        const Shell& sh = b.shells[s];
        HF_CHECK(sh.atom >= 0, HFGPU_ERR_UNSUPPORTED, "gradient needs a basis built from atoms");
        HF_CHECK(sh.L <= 2, HFGPU_ERR_UNSUPPORTED, "gradient supports s, p and d shells");
        sL[s] = sh.L; snp[s] = sh.nprim; sp0[s] = sh.prim0; sc0[s] = sh.coef0; scf[s] = sh.cfn0; sat[s] = sh.atom;
        sxyz[3 * s] = sh.x; sxyz[3 * s + 1] = sh.y; sxyz[3 * s + 2] = sh.z;
    }
    // primitive pairs grouped by L = l_A + l_B + 1 (the order of R), records consecutive per group
    constexpr int NL = 6;  // L = 1 .. 5
    std::vector<int4> items[NL];
    for (int s1 = 0; s1 < ns; ++s1)
        for (int s2 = 0; s2 <= s1; ++s2) {
            const int A = sL[s1] >= sL[s2] ? s1 : s2, B = A == s1 ? s2 : s1;
            const int L = sL[A] + sL[B] + 1;
            for (int k = 0; k < snp[A] * snp[B]; ++k) items[L].push_back(make_int4(A, B, k, 0));
        }
    std::vector<int4> all;
    int64_t off = 0;
    int64_t goff[NL + 1] = {}, gcount[NL] = {};
    for (int L = 1; L < NL; ++L) {
        goff[L] = off;
        gcount[L] = (int64_t)items[L].size();
        for (auto& it : items[L]) {
            it.w = (int)off;
            off += OG_HDR + 6 * nherm(L);
            all.push_back(it);
        }
    }
    HF_CHECK(off < ((int64_t)1 << 31), HFGPU_ERR_UNSUPPORTED, "one-electron gradient records exceed 2^31 doubles");
    std::vector<int> Z(nat);
    std::vector<double> C(3 * nat);
    for (int i = 0; i < nat; i++) {
        Z[i] = atno[i];
        for (int k = 0; k < 3; ++k) C[3 * i + k] = xyz[3 * i + k];
    }
    const size_t smem = (size_t)3 * nat * sizeof(double);
    HF_CHECK(smem <= 48 * 1024, HFGPU_ERR_UNSUPPORTED, "too many atoms for the one-electron gradient kernel");
    auto dL = to_device(sL, st);
    auto dn = to_device(snp, st);
    auto dp0 = to_device(sp0, st);
    auto dc0 = to_device(sc0, st);
    auto dcf = to_device(scf, st);
    auto dat = to_device(sat, st);
    auto dxyz = to_device(sxyz, st);
    auto dal = to_device(b.alpha, st);
    auto dco = to_device(b.coef, st);
    auto dfn = to_device(b.comp_fn, st);
    auto dit = to_device(all, st);
    auto dZ = to_device(Z, st);
    auto dC = to_device(C, st);
    DBuf<double> rec((size_t)std::max<int64_t>(off, 1), st);
    OnePairArgs o{dL.p, dn.p, dp0.p, dc0.p, dcf.p, dat.p, dxyz.p, dal.p, dco.p, dfn.p, dP, dW, n, nat,
                  dit.p, (int)all.size(), rec.p, d_grad};
    if (o.nitems > 0) {
        onee_grad_pair_kernel<<<(unsigned)((o.nitems + 127) / 128), 128, smem, st>>>(o);
        count_launch();
        HF_CUDA(cudaGetLastError());
    }
    for (int L = 1; L < NL; ++L) {
        const int64_t nth = gcount[L] * nat;
        if (nth == 0) continue;
        const unsigned blocks = (unsigned)((nth + 127) / 128);
        const double* r0 = rec.p + goff[L];
        const int nr = (int)gcount[L];
        switch (L) {
            case 1: onee_grad_nuc_kernel<1><<<blocks, 128, smem, st>>>(r0, nr, nat, dZ.p, dC.p, ctx.boys, d_grad); break;
            case 2: onee_grad_nuc_kernel<2><<<blocks, 128, smem, st>>>(r0, nr, nat, dZ.p, dC.p, ctx.boys, d_grad); break;
            case 3: onee_grad_nuc_kernel<3><<<blocks, 128, smem, st>>>(r0, nr, nat, dZ.p, dC.p, ctx.boys, d_grad); break;
            case 4: onee_grad_nuc_kernel<4><<<blocks, 128, smem, st>>>(r0, nr, nat, dZ.p, dC.p, ctx.boys, d_grad); break;
            default: onee_grad_nuc_kernel<5><<<blocks, 128, smem, st>>>(r0, nr, nat, dZ.p, dC.p, ctx.boys, d_grad); break;
        }
        count_launch();
        HF_CUDA(cudaGetLastError());
    }
}

}  // namespace hfgpu

namespace hfgpu {

__global__ void scale_occ_kernel(int n, int nocc, const double* __restrict__ C, const double* __restrict__ lam,
                                 double* __restrict__ Cs)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nocc) return;
    Cs[idx] = C[idx] * lam[idx / n];
}

void rhf_gradient(Context& ctx, EriPlan* plan, int natoms, const int* atno, const double* xyz, const double* dC,
                  const double* dL, int nocc, double* grad, double* ms_grad, double* ms_grad_eri)
{
    cudaStream_t st = ctx.stream;
    const Basis& b = plan->basis;
    const int n = b.nbf;
    const size_t nn = (size_t)n * n;
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    HF_CUDA(cudaEventRecord(e0, st));
    DBuf<double> dP(nn, st), dW(nn, st), dCs((size_t)n * std::max(nocc, 1), st), dg((size_t)3 * natoms, st);
    dg.zero();
    if (nocc > 0) {
        scale_occ_kernel<<<(unsigned)(((int64_t)n * nocc + 255) / 256), 256, 0, st>>>(n, nocc, dC, dL, dCs.p);
        count_launch();
        HF_CUDA(cudaGetLastError());
        const double two = 2.0, zero = 0.0;
        // P = 2 C_occ C_occ^T (src/scf.f90:12-24), W = 2 C_occ diag(eps) C_occ^T
        HF_CUBLAS(cublasDgemm(ctx.blas, CUBLAS_OP_N, CUBLAS_OP_T, n, n, nocc, &two, dC, n, dC, n, &zero, dP.p, n));
        HF_CUBLAS(cublasDgemm(ctx.blas, CUBLAS_OP_N, CUBLAS_OP_T, n, n, nocc, &two, dCs.p, n, dC, n, &zero, dW.p, n));
    } else {
        dP.zero();
        dW.zero();
    }
    ctx.trace_mark("grad densities");
    onee_gradient(ctx, b, natoms, atno, xyz, dP.p, dW.p, dg.p);
    ctx.trace_mark("grad one-elec");
    float ms_eri = 0;
    eri_gradient(ctx, plan, dP.p, dg.p, &ms_eri);
    ctx.trace_mark("grad two-elec");
    std::vector<double> g((size_t)3 * natoms);
    dg.download(g.data(), g.size());
    HF_CUDA(cudaEventRecord(e1, st));
    HF_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // nuclear repulsion (src/scf.f90:138-150): d/dR_i sum_{j<k} Z_j Z_k / |R_j - R_k|
    for (int i = 0; i < natoms; ++i)
        for (int j = 0; j < natoms; ++j) {
            if (i == j) continue;
            const double d[3] = {xyz[3 * i] - xyz[3 * j], xyz[3 * i + 1] - xyz[3 * j + 1], xyz[3 * i + 2] - xyz[3 * j + 2]};
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const double f = -(double)atno[i] * atno[j] / (r2 * std::sqrt(r2));
            for (int k = 0; k < 3; ++k) g[3 * i + k] += f * d[k];
        }
    for (size_t k = 0; k < g.size(); ++k) grad[k] = g[k];
    if (ms_grad) *ms_grad = ms;
    if (ms_grad_eri) *ms_grad_eri = ms_eri;
}

}  // namespace hfgpu
