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
// For each primitive quartet, with R_{tuv} the Hermite Coulomb integrals up to
// order L+1,
//   H_cd(tau)  = s_cd sum_tau' (-1)^{|tau'|} E^{cd}_tau' R_{tau+tau'}
//   T_ab(tau)  = sum_cd Gamma8_abcd H_cd(tau)
//   g_A       += s_ab sum_tau (d_A E^{ab})_tau T_ab(tau)   (and g_B the same way)
// and the mirror image for the ket centres C and D; Gamma8 = 8 Gamma.  A team of
// lanes (a power of two, picked per class) owns one shell quartet; its lanes
// split the (component pair, Hermite index) work of each primitive quartet,
// with R, H and the six density blocks of the quartet in shared memory.  The
// quartets are those the energy path evaluated (same Schwarz screening).
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
#include "internal.h"
#include "md.cuh"

namespace hfgpu {

// ------------------------------------------------------------- 1-D tables
// E[i][j][t] for i <= la+1, j <= lb+1, t <= i+j, zero elsewhere
constexpr int GE_I = 4, GE_J = 4, GE_T = 7;
constexpr int GE_DIM = GE_I * GE_J * GE_T;
constexpr int GP_HDR = 8;  // alpha_a, alpha_b, p, Px, Py, Pz, exp(-mu R_AB^2)/p, unused
constexpr int GP_STRIDE = GP_HDR + 3 * GE_DIM;
constexpr int GRAD_LMAX = 9;  // L + 1 for (dd|dd)
constexpr int GRAD_NH = nherm(GRAD_LMAX);
constexpr int GRAD_BLOCK = 128;

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
__global__ void grad_pair_kernel(const int* __restrict__ sL, const int* __restrict__ snp, const int* __restrict__ sp0,
                                 const double* __restrict__ sxyz, const double* __restrict__ alpha,
                                 const int* __restrict__ pA, const int* __restrict__ pB, const int4* __restrict__ items,
                                 int nitems, double* __restrict__ gp)
{
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nitems) return;
    const int4 item = items[it];  // (pair, record index, primitive pair within the pair)
    const int P = item.x;
    const int A = pA[P], B = pB[P];
    double* rec = gp + (int64_t)item.y * GP_STRIDE;
    const int nb = snp[B];
    const int ia = item.z / nb, ib = item.z - ia * nb;  // ia-major, as in the energy records
    const double a = alpha[sp0[A] + ia], b = alpha[sp0[B] + ib];
    const double ax = sxyz[3 * A], ay = sxyz[3 * A + 1], az = sxyz[3 * A + 2];
    const double bx = sxyz[3 * B], by = sxyz[3 * B + 1], bz = sxyz[3 * B + 2];
    const double p = a + b, ip = 1.0 / p, mu = a * b * ip;
    const double px = (a * ax + b * bx) * ip, py = (a * ay + b * by) * ip, pz = (a * az + b * bz) * ip;
    const double rab2 = (ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz);
    rec[0] = a;
    rec[1] = b;
    rec[2] = p;
    rec[3] = px;
    rec[4] = py;
    rec[5] = pz;
    rec[6] = exp(-mu * rab2) * ip;
    rec[7] = 0.0;
    const int la = sL[A] + 1, lb = sL[B] + 1;
    e1d_rt(rec + GP_HDR, la, lb, px - ax, px - bx, 0.5 * ip);
    e1d_rt(rec + GP_HDR + GE_DIM, la, lb, py - ay, py - by, 0.5 * ip);
    e1d_rt(rec + GP_HDR + 2 * GE_DIM, la, lb, pz - az, pz - bz, 0.5 * ip);
}

// Boys values F[0..M] scaled as in boys_scaled, for a runtime order M
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
struct GradArgs {
    const int* pA;
    const int* pB;
    const int* pK;
    const int* snp;
    const int* sc0;
    const int* cfn0;
    const int* comp_fn;
    const int* sat;  // atom of each shell
    const double* coef;
    const int64_t* goff;  // first record of each pair
    const double* gp;
    const double* boys;
    const int* gpairs;
    const int64_t* prefix;
    const Seg* segs;
    int nseg;
    int64_t nq;
    const int* herm;   // Hermite index -> t | u << 4 | v << 8
    const int* cartc;  // (L, component) -> l | m << 4 | n << 8
    const double* P;
    int n;
    double* grad;  // 3 per atom
    int la, lb, lc, ld;
    int team;       // lanes per quartet
    int smem_team;  // doubles of shared memory per team
};

__device__ __forceinline__ int tq(int c, int s) { return (c >> s) & 15; }

// PRIV = false: the team's lanes split each primitive quartet's component loops
// (classes with many components).  PRIV = true: each lane takes every tm-th
// primitive quartet with a private workspace, the density blocks shared (light
// classes such as (ss|ss), whose 1 - 9 components would leave most lanes idle
// while one walks up to 36 x 36 primitive quartets).
template <bool PRIV>
__global__ void __launch_bounds__(GRAD_BLOCK) eri_grad_kernel(GradArgs g)
{
    extern __shared__ double sm[];
    const int tm = g.team;
    const int tid = threadIdx.x;
    const int lt = tid & (tm - 1);
    const unsigned lane = tid & 31;
    const unsigned mask = tm == 32 ? 0xffffffffu : (((1u << tm) - 1u) << (lane & ~(unsigned)(tm - 1)));
    const int64_t qg = ((int64_t)blockIdx.x * GRAD_BLOCK + tid) / tm;
    if (qg >= g.nq) return;  // the whole team leaves together
    const int qg32 = (int)qg;
    double* ws = sm + (int64_t)(tid / tm) * g.smem_team;

    int lo = 0, hi = g.nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((int)(g.segs[mid].qoff) <= qg32) lo = mid; else hi = mid - 1;
    }
    const Seg sg = g.segs[lo];
    const int q = qg32 - (int)sg.qoff;  // class quartet counts stay below 2^31 (plan check)
    int bra, ket;
    {
        const int64_t* pf = g.prefix + sg.pref0;
        int l2 = 0, h2 = sg.nbra - 1;
        while (l2 < h2) {
            const int mid = (l2 + h2 + 1) >> 1;
            if ((int)pf[mid] <= q) l2 = mid; else h2 = mid - 1;
        }
        bra = g.gpairs[sg.bra0 + l2];
        ket = g.gpairs[sg.ket0 + (q - (int)pf[l2])];
    }
    const int A = g.pA[bra], B = g.pB[bra], C = g.pA[ket], D = g.pB[ket];
    const int la = g.la, lb = g.lb, lc = g.lc, ld = g.ld;
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const int NAB = NA * NB, NCD = NC * ND;
    const int L = la + lb + lc + ld;
    const int nHp = nherm(la + lb + 1), nHq = nherm(lc + ld + 1), nR = nherm(L + 1);

    double* PAB = ws;
    double* PCD = PAB + NAB;
    double* PAC = PCD + NCD;
    double* PBD = PAC + NA * NC;
    double* PAD = PBD + NB * ND;
    double* PBC = PAD + NA * ND;
    // per-primitive workspace: the team's, or this lane's own
    const int nshared = NAB + NCD + NA * NC + NB * ND + NA * ND + NB * NC;
    const int npriv = NAB + NCD + 2 * nR + (NCD * nHp > NAB * nHq ? NCD * nHp : NAB * nHq);
    double* sab = PBC + NB * NC + (PRIV ? lt * npriv : 0);
    double* scd = sab + NAB;
    double* R0 = scd + NCD;
    double* R1 = R0 + nR;
    double* H = R1 + nR;

    const int* fa = g.comp_fn + g.cfn0[A];
    const int* fb = g.comp_fn + g.cfn0[B];
    const int* fc = g.comp_fn + g.cfn0[C];
    const int* fd = g.comp_fn + g.cfn0[D];
    const int n = g.n;
    // component loops: split over the team, or whole in each lane
    const int c0 = PRIV ? 0 : lt, cs = PRIV ? 1 : tm;
    auto team_sync = [&]() {
        if (!PRIV) __syncwarp(mask);
    };
    auto Pv = [&](int x, int y) -> double { return (x < 0 || y < 0) ? 0.0 : __ldg(g.P + x + (int64_t)y * n); };
    for (int e = lt; e < NAB; e += tm) PAB[e] = Pv(fa[e / NB], fb[e % NB]);
    for (int e = lt; e < NCD; e += tm) PCD[e] = Pv(fc[e / ND], fd[e % ND]);
    for (int e = lt; e < NA * NC; e += tm) PAC[e] = Pv(fa[e / NC], fc[e % NC]);
    for (int e = lt; e < NB * ND; e += tm) PBD[e] = Pv(fb[e / ND], fd[e % ND]);
    for (int e = lt; e < NA * ND; e += tm) PAD[e] = Pv(fa[e / ND], fd[e % ND]);
    for (int e = lt; e < NB * NC; e += tm) PBC[e] = Pv(fb[e / NC], fc[e % NC]);
    __syncwarp(mask);

    const int kb = g.pK[bra], kk = g.pK[ket];
    const int npA = g.snp[A], npB = g.snp[B], npC = g.snp[C], npD = g.snp[D];
    const double* cA = g.coef + g.sc0[A];
    const double* cB = g.coef + g.sc0[B];
    const double* cC = g.coef + g.sc0[C];
    const double* cD = g.coef + g.sc0[D];
    const int* cla = g.cartc + la * 6;
    const int* clb = g.cartc + lb * 6;
    const int* clc = g.cartc + lc * 6;
    const int* cld = g.cartc + ld * 6;
    double gr[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) gr[k] = 0.0;

    for (int pq = PRIV ? lt : 0; pq < kb * kk; pq += PRIV ? tm : 1) {
        {
            const int pb = pq / kk, pk = pq - pb * kk;
            const double* rb = g.gp + (g.goff[bra] + pb) * GP_STRIDE;
            const double* rk = g.gp + (g.goff[ket] + pk) * GP_STRIDE;
            const double p = __ldg(rb + 2), q_ = __ldg(rk + 2);
            const double X = __ldg(rb + 3) - __ldg(rk + 3), Y = __ldg(rb + 4) - __ldg(rk + 4),
                         Z = __ldg(rb + 5) - __ldg(rk + 5);
            const double r = rsqrt_nr(p + q_);
            const double alp = p * q_ * (r * r);
            const double T = alp * (X * X + Y * Y + Z * Z);
            double F[GRAD_LMAX + 1];
            boys_rt(L + 1, T, TWO_PI_2_5 * r, -2.0 * alp, g.boys, F);
            {
                const int ia = pb / npB, ib = pb - ia * npB, ic = pk / npD, id = pk - ic * npD;
                const double kab = __ldg(rb + 6), kcd = __ldg(rk + 6);
                for (int e = c0; e < NAB; e += cs) sab[e] = cA[(e / NB) * npA + ia] * cB[(e % NB) * npB + ib] * kab;
                for (int e = c0; e < NCD; e += cs) scd[e] = cC[(e / ND) * npC + ic] * cD[(e % ND) * npD + id] * kcd;
            }
            // R^{(m)}_{tuv}, from m = L+1 down to m = 0
            double* cur = R0;
            double* nxt = R1;
            if (PRIV || lt == 0) cur[0] = F[L + 1];
            team_sync();
            for (int m = L; m >= 0; --m) {
                const int cnt = nherm(L + 1 - m);
                for (int h = c0; h < cnt; h += cs) {
                    const int c = __ldg(g.herm + h);
                    const int t = tq(c, 0), u = tq(c, 4), v = tq(c, 8);
                    double val;
                    if (h == 0) {
                        val = F[m];
                    } else if (t > 0) {
                        val = X * cur[hidx(t - 1, u, v)];
                        if (t > 1) val = fma((double)(t - 1), cur[hidx(t - 2, u, v)], val);
                    } else if (u > 0) {
                        val = Y * cur[hidx(0, u - 1, v)];
                        if (u > 1) val = fma((double)(u - 1), cur[hidx(0, u - 2, v)], val);
                    } else {
                        val = Z * cur[hidx(0, 0, v - 1)];
                        if (v > 1) val = fma((double)(v - 1), cur[hidx(0, 0, v - 2)], val);
                    }
                    nxt[h] = val;
                }
                team_sync();
                double* tmp = cur;
                cur = nxt;
                nxt = tmp;
            }
            const double* R = cur;
            const double* Bx = rb + GP_HDR;
            const double* By = Bx + GE_DIM;
            const double* Bz = By + GE_DIM;
            const double* Kx = rk + GP_HDR;
            const double* Ky = Kx + GE_DIM;
            const double* Kz = Ky + GE_DIM;

            // ---- bra centres A, B
            for (int it = c0; it < NCD * nHp; it += cs) {
                const int cd = it / nHp, h = it - cd * nHp;
                const int c = cd / ND, d = cd - c * ND;
                const int cc = clc[c], dc = cld[d], hc = __ldg(g.herm + h);
                const int cx = tq(cc, 0), cy = tq(cc, 4), cz = tq(cc, 8);
                const int dx = tq(dc, 0), dy = tq(dc, 4), dz = tq(dc, 8);
                const int t = tq(hc, 0), u = tq(hc, 4), v = tq(hc, 8);
                double acc = 0.0;
                for (int t2 = 0; t2 <= cx + dx; ++t2) {
                    const double ex = __ldg(Kx + ge(cx, dx, t2));
                    for (int u2 = 0; u2 <= cy + dy; ++u2) {
                        const double exy = ex * __ldg(Ky + ge(cy, dy, u2));
                        for (int v2 = 0; v2 <= cz + dz; ++v2) {
                            const double e = exy * __ldg(Kz + ge(cz, dz, v2));
                            const double rv = R[hidx(t + t2, u + u2, v + v2)];
                            acc = ((t2 + u2 + v2) & 1) ? fma(-e, rv, acc) : fma(e, rv, acc);
                        }
                    }
                }
                H[it] = acc * scd[cd];
            }
            team_sync();
            {
                const double al = __ldg(rb), be = __ldg(rb + 1);
                for (int it = c0; it < NAB * nHp; it += cs) {
                    const int ab = it / nHp, h = it - ab * nHp;
                    const int a = ab / NB, b = ab - a * NB;
                    const int ac = cla[a], bc = clb[b], hc = __ldg(g.herm + h);
                    const int ax = tq(ac, 0), ay = tq(ac, 4), az = tq(ac, 8);
                    const int bx = tq(bc, 0), by = tq(bc, 4), bz = tq(bc, 8);
                    const int t = tq(hc, 0), u = tq(hc, 4), v = tq(hc, 8);
                    const int ox = t - ax - bx, oy = u - ay - by, oz = v - az - bz;
                    if (ox > 1 || oy > 1 || oz > 1 || (ox > 0) + (oy > 0) + (oz > 0) > 1) continue;
                    double Tv = 0.0;
                    const double pab4 = 4.0 * PAB[ab];
                    for (int c = 0; c < NC; ++c) {
                        const double pac = PAC[a * NC + c], pbc = PBC[b * NC + c];
                        for (int d = 0; d < ND; ++d) {
                            const double gm = pab4 * PCD[c * ND + d] - pac * PBD[b * ND + d] - PAD[a * ND + d] * pbc;
                            Tv = fma(gm, H[(c * ND + d) * nHp + h], Tv);
                        }
                    }
                    const double w = sab[ab] * Tv;
                    const double ex = __ldg(Bx + ge(ax, bx, t)), ey = __ldg(By + ge(ay, by, u)),
                                 ez = __ldg(Bz + ge(az, bz, v));
                    const double dax = 2.0 * al * __ldg(Bx + ge(ax + 1, bx, t)) - (ax ? ax * __ldg(Bx + ge(ax - 1, bx, t)) : 0.0);
                    const double day = 2.0 * al * __ldg(By + ge(ay + 1, by, u)) - (ay ? ay * __ldg(By + ge(ay - 1, by, u)) : 0.0);
                    const double daz = 2.0 * al * __ldg(Bz + ge(az + 1, bz, v)) - (az ? az * __ldg(Bz + ge(az - 1, bz, v)) : 0.0);
                    const double dbx = 2.0 * be * __ldg(Bx + ge(ax, bx + 1, t)) - (bx ? bx * __ldg(Bx + ge(ax, bx - 1, t)) : 0.0);
                    const double dby = 2.0 * be * __ldg(By + ge(ay, by + 1, u)) - (by ? by * __ldg(By + ge(ay, by - 1, u)) : 0.0);
                    const double dbz = 2.0 * be * __ldg(Bz + ge(az, bz + 1, v)) - (bz ? bz * __ldg(Bz + ge(az, bz - 1, v)) : 0.0);
                    gr[0] = fma(w, dax * ey * ez, gr[0]);
                    gr[1] = fma(w, ex * day * ez, gr[1]);
                    gr[2] = fma(w, ex * ey * daz, gr[2]);
                    gr[3] = fma(w, dbx * ey * ez, gr[3]);
                    gr[4] = fma(w, ex * dby * ez, gr[4]);
                    gr[5] = fma(w, ex * ey * dbz, gr[5]);
                }
            }
            team_sync();

            // ---- ket centres C, D
            for (int it = c0; it < NAB * nHq; it += cs) {
                const int ab = it / nHq, h = it - ab * nHq;
                const int a = ab / NB, b = ab - a * NB;
                const int ac = cla[a], bc = clb[b], hc = __ldg(g.herm + h);
                const int ax = tq(ac, 0), ay = tq(ac, 4), az = tq(ac, 8);
                const int bx = tq(bc, 0), by = tq(bc, 4), bz = tq(bc, 8);
                const int t = tq(hc, 0), u = tq(hc, 4), v = tq(hc, 8);
                double acc = 0.0;
                for (int t2 = 0; t2 <= ax + bx; ++t2) {
                    const double ex = __ldg(Bx + ge(ax, bx, t2));
                    for (int u2 = 0; u2 <= ay + by; ++u2) {
                        const double exy = ex * __ldg(By + ge(ay, by, u2));
                        for (int v2 = 0; v2 <= az + bz; ++v2)
                            acc = fma(exy * __ldg(Bz + ge(az, bz, v2)), R[hidx(t + t2, u + u2, v + v2)], acc);
                    }
                }
                H[it] = ((t + u + v) & 1 ? -acc : acc) * sab[ab];
            }
            team_sync();
            {
                const double gc = __ldg(rk), gd = __ldg(rk + 1);
                for (int it = c0; it < NCD * nHq; it += cs) {
                    const int cd = it / nHq, h = it - cd * nHq;
                    const int c = cd / ND, d = cd - c * ND;
                    const int cc = clc[c], dc = cld[d], hc = __ldg(g.herm + h);
                    const int cx = tq(cc, 0), cy = tq(cc, 4), cz = tq(cc, 8);
                    const int dx = tq(dc, 0), dy = tq(dc, 4), dz = tq(dc, 8);
                    const int t = tq(hc, 0), u = tq(hc, 4), v = tq(hc, 8);
                    const int ox = t - cx - dx, oy = u - cy - dy, oz = v - cz - dz;
                    if (ox > 1 || oy > 1 || oz > 1 || (ox > 0) + (oy > 0) + (oz > 0) > 1) continue;
                    double Tv = 0.0;
                    const double pcd4 = 4.0 * PCD[cd];
                    for (int a = 0; a < NA; ++a) {
                        const double pac = PAC[a * NC + c], pad = PAD[a * ND + d];
                        for (int b = 0; b < NB; ++b) {
                            const double gm = pcd4 * PAB[a * NB + b] - pac * PBD[b * ND + d] - pad * PBC[b * NC + c];
                            Tv = fma(gm, H[(a * NB + b) * nHq + h], Tv);
                        }
                    }
                    const double w = scd[cd] * Tv;
                    const double ex = __ldg(Kx + ge(cx, dx, t)), ey = __ldg(Ky + ge(cy, dy, u)),
                                 ez = __ldg(Kz + ge(cz, dz, v));
                    const double dcx = 2.0 * gc * __ldg(Kx + ge(cx + 1, dx, t)) - (cx ? cx * __ldg(Kx + ge(cx - 1, dx, t)) : 0.0);
                    const double dcy = 2.0 * gc * __ldg(Ky + ge(cy + 1, dy, u)) - (cy ? cy * __ldg(Ky + ge(cy - 1, dy, u)) : 0.0);
                    const double dcz = 2.0 * gc * __ldg(Kz + ge(cz + 1, dz, v)) - (cz ? cz * __ldg(Kz + ge(cz - 1, dz, v)) : 0.0);
                    const double ddx = 2.0 * gd * __ldg(Kx + ge(cx, dx + 1, t)) - (dx ? dx * __ldg(Kx + ge(cx, dx - 1, t)) : 0.0);
                    const double ddy = 2.0 * gd * __ldg(Ky + ge(cy, dy + 1, u)) - (dy ? dy * __ldg(Ky + ge(cy, dy - 1, u)) : 0.0);
                    const double ddz = 2.0 * gd * __ldg(Kz + ge(cz, dz + 1, v)) - (dz ? dz * __ldg(Kz + ge(cz, dz - 1, v)) : 0.0);
                    gr[6] = fma(w, dcx * ey * ez, gr[6]);
                    gr[7] = fma(w, ex * dcy * ez, gr[7]);
                    gr[8] = fma(w, ex * ey * dcz, gr[8]);
                    gr[9] = fma(w, ddx * ey * ez, gr[9]);
                    gr[10] = fma(w, ex * ddy * ez, gr[10]);
                    gr[11] = fma(w, ex * ey * ddz, gr[11]);
                }
            }
            team_sync();
        }
    }
    for (int o = tm >> 1; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 12; ++k) gr[k] += __shfl_xor_sync(mask, gr[k], o);
    if (lt == 0) {
        const double f = (A == B ? 0.5 : 1.0) * (C == D ? 0.5 : 1.0) * (bra == ket ? 0.5 : 1.0);
        const int at[4] = {g.sat[A], g.sat[B], g.sat[C], g.sat[D]};
#pragma unroll
        for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if (gr[3 * s + k] != 0.0) atomicAdd(g.grad + 3 * at[s] + k, f * gr[3 * s + k]);
    }
}

// ------------------------------------------------------------- one-electron part
struct OneArgs {
    const int* lmn;  // 3 per function
    const int* nprim;
    const int* a0;
    const int* c0;
    const int* fatom;
    const double* xyz;  // 3 per function
    const double* alpha;
    const double* coef;
    int n, nat;
    const int* Z;
    const double* C;  // 3 per nucleus
    const double* boys;
    const double* P;
    const double* W;
    double* grad;
};

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

// nuclei per block row: the grid's second dimension splits the nuclear-attraction
// loop, so that a function pair's nuclei run in parallel (row 0 also does the
// overlap and kinetic terms)
constexpr int ONEE_GRAD_NUCLEI = 2;

__global__ void onee_grad_kernel(OneArgs o)
{
    const double PI = 3.14159265358979323846;
    extern __shared__ double sg[];  // 3 per nucleus
    for (int k = threadIdx.x; k < 3 * o.nat; k += blockDim.x) sg[k] = 0.0;
    __syncthreads();
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = o.n;
    if (idx < (int64_t)n * (n + 1) / 2) {
        int i = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
        while ((int64_t)i * (i + 1) / 2 > idx) --i;
        while ((int64_t)(i + 1) * (i + 2) / 2 <= idx) ++i;
        const int j = (int)(idx - (int64_t)i * (i + 1) / 2);
        const double sym = (i == j) ? 1.0 : 2.0;
        const double wP = sym * o.P[i + (int64_t)j * n], wW = sym * o.W[i + (int64_t)j * n];
        const int la[3] = {o.lmn[3 * i], o.lmn[3 * i + 1], o.lmn[3 * i + 2]};
        const int lb[3] = {o.lmn[3 * j], o.lmn[3 * j + 1], o.lmn[3 * j + 2]};
        const double A[3] = {o.xyz[3 * i], o.xyz[3 * i + 1], o.xyz[3 * i + 2]};
        const double B[3] = {o.xyz[3 * j], o.xyz[3 * j + 1], o.xyz[3 * j + 2]};
        const double rab2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
        double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
        double E[3][OG_I * OG_J * OG_T];
        for (int pa = 0; pa < o.nprim[i]; ++pa)
            for (int pb = 0; pb < o.nprim[j]; ++pb) {
                const double a = o.alpha[o.a0[i] + pa], b = o.alpha[o.a0[j] + pb];
                const double cc = o.coef[o.c0[i] + pa] * o.coef[o.c0[j] + pb];
                const double p = a + b, ip = 1.0 / p;
                double Pc[3];
                for (int k = 0; k < 3; ++k) {
                    Pc[k] = (a * A[k] + b * B[k]) * ip;
                    e1d_oe(E[k], la[k] + 1, lb[k] + 3, Pc[k] - A[k], Pc[k] - B[k], 0.5 * ip);
                }
                const double K = exp(-a * b * ip * rab2);
                const double pre = cc * K * PI * ip * sqrt(PI * ip);
                // 1-D overlap of powers (i, j) in direction k
                auto s1 = [&](int k, int ii, int jj) -> double { return (ii < 0 || jj < 0) ? 0.0 : E[k][og(ii, jj, 0)]; };
                // overlap and kinetic for bra powers q[] (cints.c:186-232 in 1-D overlaps)
                auto st = [&](const int* q, double& s, double& t) {
                    const double sx = s1(0, q[0], lb[0]), sy = s1(1, q[1], lb[1]), sz = s1(2, q[2], lb[2]);
                    s = sx * sy * sz;
                    double t0 = b * (2 * (lb[0] + lb[1] + lb[2]) + 3) * s;
                    double t1 = -2 * b * b *
                                (s1(0, q[0], lb[0] + 2) * sy * sz + sx * s1(1, q[1], lb[1] + 2) * sz +
                                 sx * sy * s1(2, q[2], lb[2] + 2));
                    double t2 = lb[0] * (lb[0] - 1) * s1(0, q[0], lb[0] - 2) * sy * sz +
                                lb[1] * (lb[1] - 1) * sx * s1(1, q[1], lb[1] - 2) * sz +
                                lb[2] * (lb[2] - 1) * sx * sy * s1(2, q[2], lb[2] - 2);
                    t = t0 + t1 - 0.5 * t2;
                };
                for (int k = 0; k < 3 && blockIdx.y == 0; ++k) {
                    int up[3] = {la[0], la[1], la[2]}, dn[3] = {la[0], la[1], la[2]};
                    up[k] += 1;
                    dn[k] -= 1;
                    double su, tu, sd = 0, td = 0;
                    st(up, su, tu);
                    if (la[k] > 0) st(dn, sd, td);
                    const double dS = pre * (2 * a * su - la[k] * sd);
                    const double dT = pre * (2 * a * tu - la[k] * td);
                    const double gk = wP * dT - wW * dS;
                    gA[k] += gk;  // two-centre: d/dB = -d/dA
                    gB[k] -= gk;
                }
                // nuclear attraction
                const int L = la[0] + la[1] + la[2] + lb[0] + lb[1] + lb[2] + 1;
                const double vpre = wP * cc * K * 2 * PI * ip;
                const int c_end = min(o.nat, (int)(blockIdx.y + 1) * ONEE_GRAD_NUCLEI);
                for (int c = blockIdx.y * ONEE_GRAD_NUCLEI; c < c_end; ++c) {
                    const double X = Pc[0] - o.C[3 * c], Y = Pc[1] - o.C[3 * c + 1], Zc = Pc[2] - o.C[3 * c + 2];
                    double F[OG_L + 1];
                    boys_rt(L, p * (X * X + Y * Y + Zc * Zc), 1.0, -2.0 * p, o.boys, F);
                    double R[OG_L + 1][nherm(OG_L)];
                    for (int m = 0; m <= L; ++m) R[m][0] = F[m];
                    for (int m = L - 1; m >= 0; --m)
                        for (int s = 1; s <= L - m; ++s)
                            for (int t = s; t >= 0; --t)
                                for (int v = 0; v <= s - t; ++v) {
                                    const int u = s - t - v;
                                    double r;
                                    if (t > 0) {
                                        r = X * R[m + 1][hidx(t - 1, u, v)];
                                        if (t > 1) r = fma((double)(t - 1), R[m + 1][hidx(t - 2, u, v)], r);
                                    } else if (u > 0) {
                                        r = Y * R[m + 1][hidx(0, u - 1, v)];
                                        if (u > 1) r = fma((double)(u - 1), R[m + 1][hidx(0, u - 2, v)], r);
                                    } else {
                                        r = Zc * R[m + 1][hidx(0, 0, v - 1)];
                                        if (v > 1) r = fma((double)(v - 1), R[m + 1][hidx(0, 0, v - 2)], r);
                                    }
                                    R[m][hidx(t, u, v)] = r;
                                }
                    // Hermite sum for bra powers q[] and ket powers w[]
                    auto hs = [&](const int* q, const int* w) -> double {
                        if (q[0] < 0 || q[1] < 0 || q[2] < 0 || w[0] < 0 || w[1] < 0 || w[2] < 0) return 0.0;
                        double acc = 0;
                        for (int t = 0; t <= q[0] + w[0]; ++t)
                            for (int u = 0; u <= q[1] + w[1]; ++u)
                                for (int v = 0; v <= q[2] + w[2]; ++v)
                                    acc += E[0][og(q[0], w[0], t)] * E[1][og(q[1], w[1], u)] * E[2][og(q[2], w[2], v)] *
                                           R[0][hidx(t, u, v)];
                        return acc;
                    };
                    const double zc = -(double)o.Z[c] * vpre;
                    double hc[3];
                    for (int k = 0; k < 3; ++k) {
                        int up[3] = {la[0], la[1], la[2]}, dn[3] = {la[0], la[1], la[2]};
                        up[k] += 1;
                        dn[k] -= 1;
                        const double dA = zc * (2 * a * hs(up, lb) - la[k] * hs(dn, lb));
                        int ub[3] = {lb[0], lb[1], lb[2]}, db[3] = {lb[0], lb[1], lb[2]};
                        ub[k] += 1;
                        db[k] -= 1;
                        const double dB = zc * (2 * b * hs(la, ub) - lb[k] * hs(la, db));
                        gA[k] += dA;
                        gB[k] += dB;
                        hc[k] = -(dA + dB);  // Hellmann-Feynman term of nucleus c
                    }
                    for (int k = 0; k < 3; ++k)
                        if (hc[k] != 0.0) atomicAdd(sg + 3 * c + k, hc[k]);
                }
            }
        const int ai = o.fatom[i], aj = o.fatom[j];
        for (int k = 0; k < 3; ++k) {
            atomicAdd(sg + 3 * ai + k, gA[k]);
            atomicAdd(sg + 3 * aj + k, gB[k]);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * o.nat; k += blockDim.x)
        if (sg[k] != 0.0) atomicAdd(o.grad + k, sg[k]);
}

// ------------------------------------------------------------- host side
static int grad_team(int la, int lb, int lc, int ld)
{
    const int w = ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) *
                  std::max(nherm(la + lb + 1), nherm(lc + ld + 1));
    if (w >= 2000) return 32;
    if (w >= 500) return 16;
    if (w >= 120) return 8;
    return 4;
}

// classes with at most this many component quartets run the primitive loop one
// primitive quartet per lane (eri_grad_kernel<true>), 8 lanes per shell quartet
constexpr int GRAD_PRIV_MAX = 9, GRAD_PRIV_TEAM = 8;

static bool grad_priv(int la, int lb, int lc, int ld)
{
    return ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) <= GRAD_PRIV_MAX;
}

// doubles of shared memory per team: the six density blocks, then the
// per-primitive workspace (one per lane in the private mode)
static int grad_smem_team(int la, int lb, int lc, int ld, bool priv, int team)
{
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const int NAB = NA * NB, NCD = NC * ND;
    const int nHp = nherm(la + lb + 1), nHq = nherm(lc + ld + 1), nR = nherm(la + lb + lc + ld + 1);
    const int shared = NAB + NCD + NA * NC + NB * ND + NA * ND + NB * NC;
    const int work = NAB + NCD + 2 * nR + std::max(NCD * nHp, NAB * nHq);
    return shared + (priv ? team : 1) * work;
}

void eri_gradient(Context& ctx, EriPlan* P, const double* dP, double* d_grad, float* ms_out)
{
    cudaStream_t st = ctx.stream;
    const Basis& b = P->basis;
    const int ns = (int)b.shells.size();
    std::vector<int> sat(ns);
    for (int s = 0; s < ns; ++s) {
        HF_CHECK(b.shells[s].atom >= 0, HFGPU_ERR_UNSUPPORTED, "gradient needs a basis built from atoms");
        HF_CHECK(b.shells[s].L <= 2, HFGPU_ERR_UNSUPPORTED, "gradient supports s, p and d shells");
        sat[s] = b.shells[s].atom;
    }
    // gradient pair records: pair P's records are consecutive, (ia, ib) ia-major
    std::vector<int64_t> goff(P->npair);
    std::vector<int4> items;
    int64_t nrec = 0;
    for (int id = 0; id < P->npair; ++id) {
        goff[id] = nrec;
        for (int k = 0; k < P->pK[id]; ++k) items.push_back(make_int4(id, (int)(nrec + k), k, 0));
        nrec += P->pK[id];
    }
    DBuf<double> gp((size_t)nrec * GP_STRIDE, st);
    DBuf<int4> dit = to_device(items, st);
    {
        const int ni = (int)items.size();
        grad_pair_kernel<<<(ni + 127) / 128, 128, 0, st>>>(P->sL.p, P->snp.p, P->sp0.p, P->sxyz.p, P->alpha.p,
                                                          P->dA.p, P->dB.p, dit.p, ni, gp.p);
        count_launch();
        HF_CUDA(cudaGetLastError());
    }
    std::vector<int> herm(GRAD_NH), cartc(3 * 6, 0);
    for (int s = 0; s <= GRAD_LMAX; ++s)
        for (int w = 0; w <= s; ++w)
            for (int v = 0; v <= w; ++v) {
                const int u = w - v, t = s - w;
                herm[hidx(t, u, v)] = t | (u << 4) | (v << 8);
            }
    for (int L = 0; L <= 2; ++L)
        for (int c = 0; c < ncart(L); ++c) {
            const Cart cc = cart(L, c);
            cartc[L * 6 + c] = cc.l | (cc.m << 4) | (cc.n << 8);
        }
    DBuf<int> dherm = to_device(herm, st), dcart = to_device(cartc, st), dsat = to_device(sat, st);
    DBuf<int64_t> dgoff = to_device(goff, st);

    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(eri_grad_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(eri_grad_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    ctx.trace_mark("grad pair data");
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    HF_CUDA(cudaEventRecord(e0, st));
    for (int i = (int)P->classes.size() - 1; i >= 0; --i) {
        const ClassPlan& c = P->classes[i];
        if (c.nq == 0) continue;
        GradArgs a;
        a.pA = P->dA.p; a.pB = P->dB.p; a.pK = P->dK.p;
        a.snp = P->snp.p; a.sc0 = P->sc0.p; a.cfn0 = P->scf.p; a.comp_fn = P->cfn.p;
        a.sat = dsat.p; a.coef = P->coef.p;
        a.goff = dgoff.p; a.gp = gp.p; a.boys = ctx.boys;
        a.gpairs = P->gpairs.p; a.prefix = P->prefix.p;
        a.segs = c.dsegs.p; a.nseg = (int)c.segs.size(); a.nq = c.nq;
        a.herm = dherm.p; a.cartc = dcart.p;
        a.P = dP; a.n = b.nbf; a.grad = d_grad;
        a.la = ptype_la(c.tb); a.lb = ptype_lb(c.tb); a.lc = ptype_la(c.tk); a.ld = ptype_lb(c.tk);
        const bool priv = grad_priv(a.la, a.lb, a.lc, a.ld);
        int team = priv ? GRAD_PRIV_TEAM : grad_team(a.la, a.lb, a.lc, a.ld);
        int smt = grad_smem_team(a.la, a.lb, a.lc, a.ld, priv, team);
        while (!priv && team < 32 && (size_t)(GRAD_BLOCK / team) * smt * sizeof(double) > 200 * 1024) team <<= 1;
        const size_t smem = (size_t)(GRAD_BLOCK / team) * smt * sizeof(double);
        HF_CHECK(smem <= 200 * 1024, HFGPU_ERR_UNSUPPORTED, "gradient workspace exceeds shared memory");
        a.team = team;
        a.smem_team = smt;
        const int64_t blocks = (c.nq * team + GRAD_BLOCK - 1) / GRAD_BLOCK;
        if (priv) eri_grad_kernel<true><<<(unsigned)blocks, GRAD_BLOCK, smem, st>>>(a);
        else eri_grad_kernel<false><<<(unsigned)blocks, GRAD_BLOCK, smem, st>>>(a);
        count_launch();
        HF_CUDA(cudaGetLastError());
    }
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
    std::vector<int> lmn(3 * n), np(n), a0(n), c0(n), fat(n);
    std::vector<double> fx(3 * n);
    for (auto& sh : b.shells) {
        HF_CHECK(sh.atom >= 0, HFGPU_ERR_UNSUPPORTED, "gradient needs a basis built from atoms");
        for (int c = 0; c < ncart(sh.L); c++) {
            const int fn = b.comp_fn[sh.cfn0 + c];
            if (fn < 0) continue;
            const Cart cc = cart(sh.L, c);
            lmn[3 * fn] = cc.l; lmn[3 * fn + 1] = cc.m; lmn[3 * fn + 2] = cc.n;
            np[fn] = sh.nprim;
            a0[fn] = sh.prim0;
            c0[fn] = sh.coef0 + c * sh.nprim;
            fat[fn] = sh.atom;
            fx[3 * fn] = sh.x; fx[3 * fn + 1] = sh.y; fx[3 * fn + 2] = sh.z;
        }
    }
    std::vector<int> Z(nat);
    std::vector<double> C(3 * nat);
    for (int i = 0; i < nat; i++) {
        Z[i] = atno[i];
        for (int k = 0; k < 3; ++k) C[3 * i + k] = xyz[3 * i + k];
    }
    auto dl = to_device(lmn, st);
    auto dn = to_device(np, st);
    auto da = to_device(a0, st);
    auto dc = to_device(c0, st);
    auto dfa = to_device(fat, st);
    auto dx = to_device(fx, st);
    auto dal = to_device(b.alpha, st);
    auto dco = to_device(b.coef, st);
    auto dZ = to_device(Z, st);
    auto dC = to_device(C, st);
    OneArgs o{dl.p, dn.p, da.p, dc.p, dfa.p, dx.p, dal.p, dco.p, n, nat, dZ.p, dC.p, ctx.boys, dP, dW, d_grad};
    const int64_t npair = (int64_t)n * (n + 1) / 2;
    const size_t smem = (size_t)3 * nat * sizeof(double);
    HF_CHECK(smem <= 48 * 1024, HFGPU_ERR_UNSUPPORTED, "too many atoms for the one-electron gradient kernel");
    const dim3 grid((unsigned)((npair + 127) / 128), (unsigned)((nat + ONEE_GRAD_NUCLEI - 1) / ONEE_GRAD_NUCLEI));
    onee_grad_kernel<<<grid, 128, smem, st>>>(o);
    count_launch();
    HF_CUDA(cudaGetLastError());
    HF_CUDA(cudaStreamSynchronize(st));
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
                  const double* dL, int nocc, double* grad, double* ms_grad)
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
    eri_gradient(ctx, plan, dP.p, dg.p, nullptr);
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
}

}  // namespace hfgpu
