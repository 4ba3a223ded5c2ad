// ERI gradient class kernel: the part shared by all ordered quartet classes.
// The class-specific arithmetic (GradPrim: one primitive quartet's ket sums;
// GradContract: the density contraction of one bra primitive pair) is
// generated by gen_grad.py into gen/grad_class_<TB><TK>.cu.
//
// For a quartet (bra | ket) of screened shell pairs, a thread owns the ket
// component pairs of one chunk and every bra component pair.  Its `split`
// lanes take the bra primitive pairs in turn (and slices of the ket primitive
// pairs when there are more lanes than bra primitives); for each one the ket
// primitive pairs are summed into the Hermite accumulators X first, then X is
// contracted with
//     Gamma8_{ab,cd} = 4 P_ab P_cd - P_ac P_bd - P_ad P_bc
// (eight times the two-particle density of a closed shell) and the bra
// pair's derivative coefficients.  The result is the derivative of
//     f sum_{ab,cd} Gamma8_{ab,cd} (ab|cd),  f = 1/2 per coincident pair and
//     for bra == ket (the multiplicity of the unique quartet),
// with respect to the bra's first centre (gA) and, for WITHP, to both bra
// centres moved together (gP).  By translational invariance the kernel with
// WITHP credits A with gA, B with gP - gA and the ket's second centre D with
// -gP; the swapped launch credits the ket's first centre C with its own gA
// and D with -gA, so D ends with -(gP + gC), the remaining component.
#pragma once
#include <cstdint>

#include "boys.cuh"
#include "eri_kernel.cuh"
#include "md.cuh"

namespace hfgpu {

constexpr int GR_HDR = 20;  // alpha, beta, p, Px, Py, Pz, K_ab, unused, c_a K_ab (6), c_b (6)
constexpr int GRAD_XCAP = 48;
constexpr int GRAD_BLK = 128;

HD constexpr int grad_table(int la, int lb) { return (la + 1) * (lb + 1) * (la + lb + 2); }
HD constexpr int grad_stride(int la, int lb) { return GR_HDR + 6 * grad_table(la, lb); }

HD constexpr int grad_ncd(int tb, int tk)
{
    const int nh1 = nherm(ptype_la(tb) + ptype_lb(tb) + 1);
    const int ncdt = ncart(ptype_la(tk)) * ncart(ptype_lb(tk));
    for (int n = ncdt; n >= 1; --n)
        if (ncdt % n == 0 && n * nh1 <= GRAD_XCAP) return n;
    return 1;
}

template <int TB, int TK>
struct GradInfo {
    static constexpr int LA = ptype_la(TB), LB = ptype_lb(TB), LC = ptype_la(TK), LD = ptype_lb(TK);
    static constexpr int L = LA + LB + LC + LD;
    static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    static constexpr int NAB = NA * NB, NCDT = NC * ND;
    static constexpr int NH1 = nherm(LA + LB + 1);
    static constexpr int NCDC = grad_ncd(TB, TK), G = NCDT / NCDC;
    static constexpr int SK = pair_stride(LC, LD);  // ket: energy pair record
    static constexpr int SG = grad_stride(LA, LB);  // bra: gradient pair record
    static constexpr int GAM = NAB * NCDC;          // density values per thread
};

struct GradArgs {
    const int* pA;
    const int* pB;
    const int* pK;
    const int64_t* poff;  // energy pair records (ket side)
    const double* pdata;
    const int64_t* goff;  // gradient pair records (bra side)
    const double* gdata;
    const double* boys;
    const int* gpairs;
    const int64_t* prefix;
    const Seg* segs;  // the class's segments, warp0 and split laid out for this launch
    int nseg;
    int64_t nwarps;
    const int* cfn0;
    const int* comp_fn;
    const int* sat;  // atom of each shell
    const double* P;
    int n;
    int nat;
    int gam_stride;  // doubles of density storage per thread slot (the largest GAM of the launch)
    double* grad;    // 3 per atom
};

using GradKernelFn = void (*)(GradArgs);

template <int TB, int TK, int CH>
struct GradPrim;  // generated
template <int TB, bool WITHP>
struct GradContract;  // generated

// the ket sums of one primitive quartet for the warp's chunk (warp-uniform)
template <int TB, int TK, int G, int CH>
__device__ __forceinline__ void grad_prim_dispatch(int chunk, double (&acc)[GradInfo<TB, TK>::NCDC * GradInfo<TB, TK>::NH1],
                                                   const double* ek, const double (&F)[GradInfo<TB, TK>::L + 2],
                                                   double X, double Y, double Z)
{
    if constexpr (CH < G) {
        if (chunk == CH)
            GradPrim<TB, TK, CH>::prim(acc, ek, F, X, Y, Z);
        else
            grad_prim_dispatch<TB, TK, G, CH + 1>(chunk, acc, ek, F, X, Y, Z);
    }
}

template <int TB, int TK, bool WITHP>
__device__ __forceinline__ void grad_quartet(const GradArgs& a, int chunk, double* gam, double* sgrad, int bra,
                                             int ket, bool active, int sub, int split)
{
    using GI = GradInfo<TB, TK>;
    const int A = a.pA[bra], B = a.pB[bra], C = a.pA[ket], D = a.pB[ket];
    {
        const int* fa = a.comp_fn + a.cfn0[A];
        const int* fb = a.comp_fn + a.cfn0[B];
        const int* fc = a.comp_fn + a.cfn0[C];
        const int* fd = a.comp_fn + a.cfn0[D];
        const int n = a.n;
        auto Pv = [&](int x, int y) -> double { return (x < 0 || y < 0) ? 0.0 : __ldg(a.P + x + (int64_t)y * n); };
        for (int ab = 0; ab < GI::NAB; ++ab) {
            const int i = fa[ab / GI::NB], j = fb[ab % GI::NB];
#pragma unroll
            for (int s = 0; s < GI::NCDC; ++s) {
                const int cd = chunk * GI::NCDC + s;
                const int k = fc[cd / GI::ND], l = fd[cd % GI::ND];
                gam[(ab * GI::NCDC + s) * GRAD_BLK] =
                    4.0 * Pv(i, j) * Pv(k, l) - Pv(i, k) * Pv(j, l) - Pv(i, l) * Pv(j, k);
            }
        }
    }
    double g[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int kb = a.pK[bra], kk = a.pK[ket];
    const double* rb0 = a.gdata + a.goff[bra];
    const double* rk0 = a.pdata + a.poff[ket];
    // work items (bra primitive pair, slice of the ket primitive pairs): with
    // more lanes than bra primitives, the ket primitives are dealt out too
    // (the contraction is linear in X, so each slice is contracted on its own)
    const int nkc = split > kb ? (split + kb - 1) / kb : 1;
    for (int it = sub; it < kb * nkc; it += split) {
        const int pb = it / nkc, kc = it - pb * nkc;
        const double* rb = rb0 + (int64_t)pb * GI::SG;
        const double p = __ldg(rb + 2), px = __ldg(rb + 3), py = __ldg(rb + 4), pz = __ldg(rb + 5);
        double acc[GI::NCDC * GI::NH1];
#pragma unroll
        for (int i = 0; i < GI::NCDC * GI::NH1; ++i) acc[i] = 0.0;
        for (int pk = kc; pk < kk; pk += nkc) {
            const double* rk = rk0 + (int64_t)pk * GI::SK;
            const double q = __ldg(rk), qx = __ldg(rk + 1), qy = __ldg(rk + 2), qz = __ldg(rk + 3);
            const double r = rsqrt_nr(p + q);
            const double alpha = p * q * (r * r);
            const double X = px - qx, Y = py - qy, Z = pz - qz;
            const double T = alpha * (X * X + Y * Y + Z * Z);
            double F[GI::L + 2];
            boys_scaled<GI::L + 1>(T, TWO_PI_2_5 * r, -2.0 * alpha, a.boys, F);
            grad_prim_dispatch<TB, TK, GI::G, 0>(chunk, acc, rk + PAIR_HDR, F, X, Y, Z);
        }
#pragma unroll
        for (int s = 0; s < GI::NCDC; ++s)
            GradContract<TB, WITHP>::template run<GI::NCDC * GRAD_BLK>(acc + s * GI::NH1, gam + s * GRAD_BLK, rb, g);
    }
    if (split > 1) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
            for (int o = split >> 1; o > 0; o >>= 1) g[k] += __shfl_xor_sync(0xffffffffu, g[k], o);
    }
    if (!active || sub != 0) return;
    const double f = (A == B ? 0.5 : 1.0) * (C == D ? 0.5 : 1.0) * (bra == ket ? 0.5 : 1.0);
    const int ta = 3 * a.sat[A], tb_ = 3 * a.sat[B], td = 3 * a.sat[D];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (WITHP) {
            atomicAdd(sgrad + ta + k, f * g[k]);
            atomicAdd(sgrad + tb_ + k, f * (g[3 + k] - g[k]));
            atomicAdd(sgrad + td + k, -f * g[3 + k]);
        } else {
            atomicAdd(sgrad + ta + k, f * g[k]);
            atomicAdd(sgrad + tb_ + k, -f * g[k]);
        }
    }
}

// One warp = 32/split quartets of one segment for one ket chunk.  SWAP: the
// segment's quartets are (bra | ket) of the energy class (TK, TB); this launch
// differentiates their ket, so the pairs trade places.  Dynamic shared memory:
// the density values of every thread, then the block's gradient (3 per atom),
// which is added to the output once per block.
template <int TB, int TK, bool WITHP, bool SWAP>
__global__ void __launch_bounds__(GRAD_BLK) grad_class_kernel(GradArgs a)
{
    using GI = GradInfo<TB, TK>;
    extern __shared__ double gsm[];
    double* sgrad = gsm + (int64_t)a.gam_stride * GRAD_BLK;
    for (int k = threadIdx.x; k < 3 * a.nat; k += GRAD_BLK) sgrad[k] = 0.0;
    __syncthreads();
    const int w = blockIdx.x * (GRAD_BLK / 32) + threadIdx.x / 32;
    if (w < (int)a.nwarps) {
        const int lane = threadIdx.x & 31;
        int lo = 0, hi = a.nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((int)a.segs[mid].warp0 <= w) lo = mid; else hi = mid - 1;
        }
        const Seg sg = a.segs[lo];
        const int lw = w - (int)sg.warp0;
        const int chunk = lw % GI::G;
        const int split = sg.split;
        const int sub = lane & (split - 1);
        int q = (lw / GI::G) * (32 / split) + lane / split;
        const bool active = q < (int)sg.nq;
        if (!active) q = (int)sg.nq - 1;
        const int64_t* pf = a.prefix + sg.pref0;
        int l2 = 0, h2 = sg.nbra - 1;
        while (l2 < h2) {
            const int mid = (l2 + h2 + 1) >> 1;
            if ((int)pf[mid] <= q) l2 = mid; else h2 = mid - 1;
        }
        int bra = a.gpairs[sg.bra0 + l2];
        int ket = a.gpairs[sg.ket0 + (q - (int)pf[l2])];
        if (SWAP) {
            const int t = bra;
            bra = ket;
            ket = t;
        }
        grad_quartet<TB, TK, WITHP>(a, chunk, gsm + threadIdx.x, sgrad, bra, ket, active, sub, split);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * a.nat; k += GRAD_BLK)
        if (sgrad[k] != 0.0) atomicAdd(a.grad + k, sgrad[k]);
}

// the launches an ordered class takes part in: (TB, TK) with TB <= TK is the
// bra side of energy class (TB, TK); TB >= TK is the swapped side of (TK, TB)
template <int TB, int TK>
GradKernelFn select_grad_kernel(bool withp)
{
    if constexpr (TB < TK) {
        return withp ? grad_class_kernel<TB, TK, true, false> : nullptr;
    } else if constexpr (TB > TK) {
        return withp ? nullptr : grad_class_kernel<TB, TK, false, true>;
    } else {
        return withp ? grad_class_kernel<TB, TK, true, false> : grad_class_kernel<TB, TK, false, true>;
    }
}

}  // namespace hfgpu
