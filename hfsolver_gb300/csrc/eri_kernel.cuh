// ERI class kernel: the part shared by all quartet classes.  The class-specific
// arithmetic of one primitive quartet (EriBody<TB, TK, CH>::prim) is generated
// by gen_eri.py into gen/eri_class_<TB><TK>.cu, one translation unit per class.
#pragma once
#include <cstdint>

#include "boys.cuh"
#include "md.cuh"

namespace hfgpu {

struct ShellDev {
    const int* L;
    const int* nprim;
    const double* xyz;  // 3 per shell
    const int* prim0;
    const int* coef0;
    const int* cfn0;
    const double* alpha;
    const double* coef;
    const int* comp_fn;
};

struct PairDev {
    const int* A;        // shell with the larger L first
    const int* B;
    const int* K;        // primitive pairs
    const int64_t* off;  // offset of the first record in pdata
    const double* pdata;
};

// A run of quartets of one class whose bra pairs come from one group and ket
// pairs from another (each group: one pair type and one primitive count).
struct Seg {
    int64_t warp0;   // first warp of the segment within its class launch
    int64_t nq;      // quartets
    int64_t pref0;   // prefix-sum offset (prefix mode) or list offset (list mode)
    int64_t qoff;    // index of the segment's first quartet within its class
    int bra0, ket0;  // offsets into the grouped, sorted pair-id array
    int nbra;
    int list;        // 1: explicit (bra, ket) list
    int split;       // lanes per quartet (power of two): they share its primitive pairs
    int mol;         // molecule of the segment in a batched plan (0 for one molecule)
};

enum { MODE_PACKED = 0, MODE_DIAG = 1 };

struct EriArgs {
    ShellDev sh;
    PairDev pr;
    const double* boys;
    const int* gpairs;      // pair ids, grouped and sorted
    const int64_t* prefix;  // per segment: nbra+1 prefix sums of ket counts
    const int2* list;       // list-mode quartets (pair ids)
    const Seg* segs;
    int nseg;
    int64_t nwarps;
    double* out;     // packed integrals (may be null), or diagonal buffer [pair][36]
    double* blocks;  // class-wise quartet blocks [element][quartet] (may be null)
    int64_t nq_class;
    const int64_t* mol_out;  // batched plans: offset of each molecule's packed array in out (else null)
    int2* qlist;             // with blocks: the (bra, ket) pair ids of each quartet of the class (else null)
};

using KernelFn = void (*)(EriArgs);

constexpr int ERI_BLOCK = 128;
constexpr double TWO_PI_2_5 = 34.986836655249725;  // 2 pi^{5/2}

__host__ __device__ constexpr int pick_ncd(int nab, int ncd)
{
    for (int n = ncd; n >= 1; --n)
        if (ncd % n == 0 && nab * n <= 36) return n;
    return 1;
}

template <int TB, int TK>
struct ClassInfo {
    static constexpr int LA = ptype_la(TB), LB = ptype_lb(TB), LC = ptype_la(TK), LD = ptype_lb(TK);
    static constexpr int L = LA + LB + LC + LD;
    static constexpr int NAB = ncart(LA) * ncart(LB), NCDT = ncart(LC) * ncart(LD);
    static constexpr int NCD = pick_ncd(NAB, NCDT), G = NCDT / NCD;
    static constexpr int SB = pair_stride(LA, LB), SK = pair_stride(LC, LD);
};

template <int TB, int TK, int CH>
struct EriBody;  // generated

template <int TB, int TK, int MODE, int CH>
__device__ __forceinline__ void run_chunk(const EriArgs& a, double* out, int bra, int ket, bool active, int64_t qg,
                                          int sub, int split)
{
    using CI = ClassInfo<TB, TK>;
    double acc[CI::NAB * CI::NCD];
#pragma unroll
    for (int i = 0; i < CI::NAB * CI::NCD; ++i) acc[i] = 0.0;
    const int kb = a.pr.K[bra], kk = a.pr.K[ket];
    const double* pb0 = a.pr.pdata + a.pr.off[bra];
    const double* pk0 = a.pr.pdata + a.pr.off[ket];
    // the split lanes of a quartet take its primitive pairs in turn
    for (int pp = sub; pp < kb * kk; pp += split) {
        const int ib = pp / kk, ik = pp - ib * kk;
        const double* pb = pb0 + (int64_t)ib * CI::SB;
        const double* pk = pk0 + (int64_t)ik * CI::SK;
        const double p = __ldg(pb), px = __ldg(pb + 1), py = __ldg(pb + 2), pz = __ldg(pb + 3);
        const double q = __ldg(pk), qx = __ldg(pk + 1), qy = __ldg(pk + 2), qz = __ldg(pk + 3);
        const double r = rsqrt_nr(p + q);
        const double alpha = p * q * (r * r);
        const double X = px - qx, Y = py - qy, Z = pz - qz;
        const double T = alpha * (X * X + Y * Y + Z * Z);
        double F[CI::L + 1];
        boys_scaled<CI::L>(T, TWO_PI_2_5 * r, -2.0 * alpha, a.boys, F);
        EriBody<TB, TK, CH>::prim(acc, pb + PAIR_HDR, pk + PAIR_HDR, F, X, Y, Z);
    }
    if (split > 1) {  // sum the partial accumulators of the split lanes (aligned groups)
#pragma unroll
        for (int i = 0; i < CI::NAB * CI::NCD; ++i)
            for (int o = split >> 1; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
    }
    if (!active || sub != 0) return;
    if constexpr (MODE == MODE_DIAG) {
        // bra == ket: keep the diagonal values (ab|ab) for the Schwarz bound
#pragma unroll
        for (int s = 0; s < CI::NCD; ++s) {
            const int icd = CH * CI::NCD + s;
            out[(int64_t)ket * 36 + icd] = acc[icd * CI::NCD + s];
        }
    } else {
        if (a.qlist && CH == 0) a.qlist[qg] = make_int2(bra, ket);
        if (a.blocks) {  // the whole block, one element plane per component quartet (coalesced in q)
#pragma unroll
            for (int s = 0; s < CI::NCD; ++s)
#pragma unroll
                for (int ab = 0; ab < CI::NAB; ++ab)
                    a.blocks[(int64_t)(ab * CI::NCDT + CH * CI::NCD + s) * a.nq_class + qg] = acc[ab * CI::NCD + s];
        }
        if (!out) return;
        const int A = a.pr.A[bra], B = a.pr.B[bra], C = a.pr.A[ket], D = a.pr.B[ket];
        const int* fa = a.sh.comp_fn + a.sh.cfn0[A];
        const int* fb = a.sh.comp_fn + a.sh.cfn0[B];
        const int* fc = a.sh.comp_fn + a.sh.cfn0[C];
        const int* fd = a.sh.comp_fn + a.sh.cfn0[D];
        const bool sameAB = (A == B), sameCD = (C == D), sameBK = (bra == ket);
#pragma unroll
        for (int s = 0; s < CI::NCD; ++s) {
            const int icd = CH * CI::NCD + s;
            const int k = fc[icd / ncart(CI::LD)], l = fd[icd % ncart(CI::LD)];
            if (k < 0 || l < 0 || (sameCD && k < l)) continue;
            const int kh = k > l ? k : l, kl = kh * (kh + 1) / 2 + (k > l ? l : k);
#pragma unroll
            for (int ab = 0; ab < CI::NAB; ++ab) {
                const int i = fa[ab / ncart(CI::LB)], j = fb[ab % ncart(CI::LB)];
                if (i < 0 || j < 0 || (sameAB && i < j)) continue;
                const int ih = i > j ? i : j, ij = ih * (ih + 1) / 2 + (i > j ? j : i);
                if (sameBK && ij < kl) continue;
                // pair indices fit 32 bits (n <= 512); only the packed position needs 64
                const int64_t idx = ij >= kl ? (((int64_t)ij * (ij + 1)) >> 1) + kl : (((int64_t)kl * (kl + 1)) >> 1) + ij;
                out[idx] = acc[ab * CI::NCD + s];
            }
        }
    }
}

template <int TB, int TK, int MODE, int G, int CH>
__device__ __forceinline__ void dispatch_chunk(const EriArgs& a, double* out, int chunk, int bra, int ket, bool active,
                                               int64_t qg, int sub, int split)
{
    if constexpr (CH < G) {
        if (chunk == CH)
            run_chunk<TB, TK, MODE, CH>(a, out, bra, ket, active, qg, sub, split);
        else
            dispatch_chunk<TB, TK, MODE, G, CH + 1>(a, out, chunk, bra, ket, active, qg, sub, split);
    }
}

// One warp = 32/split quartets of one segment for one ket chunk (warp-uniform);
// split lanes share each quartet's primitive pairs.
template <int TB, int TK, int MODE>
__global__ void __launch_bounds__(ERI_BLOCK) eri_class_kernel(EriArgs a)
{
    using CI = ClassInfo<TB, TK>;
    // warp, quartet and prefix-sum values of a class stay below 2^31 (checked when
    // the plan is made): the searches compare in 32 bits (64-bit compares run on
    // this GPU's narrow FP64 pipe, which the integrals need)
    const int w = blockIdx.x * (ERI_BLOCK / 32) + threadIdx.x / 32;
    if (w >= (int)a.nwarps) return;
    const int lane = threadIdx.x & 31;
    int lo = 0, hi = a.nseg - 1;  // last segment with warp0 <= w
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((int)a.segs[mid].warp0 <= w) lo = mid; else hi = mid - 1;
    }
    const Seg sg = a.segs[lo];
    const int lw = w - (int)sg.warp0;
    const int chunk = lw % CI::G;
    const int split = sg.split;
    const int sub = lane & (split - 1);
    int q = (lw / CI::G) * (32 / split) + lane / split;
    const bool active = q < (int)sg.nq;
    if (!active) q = (int)sg.nq - 1;
    int bra, ket;
    if (sg.list) {
        const int2 e = a.list[sg.pref0 + q];
        bra = e.x;
        ket = e.y;
    } else {
        const int64_t* pf = a.prefix + sg.pref0;
        int l2 = 0, h2 = sg.nbra - 1;  // last bra i with pf[i] <= q
        while (l2 < h2) {
            const int mid = (l2 + h2 + 1) >> 1;
            if ((int)pf[mid] <= q) l2 = mid; else h2 = mid - 1;
        }
        bra = a.gpairs[sg.bra0 + l2];
        ket = a.gpairs[sg.ket0 + (q - (int)pf[l2])];
    }
    double* out = a.out;
    if (out && a.mol_out) out += a.mol_out[sg.mol];  // the segment's molecule's packed array
    dispatch_chunk<TB, TK, MODE, CI::G, 0>(a, out, chunk, bra, ket, active, sg.qoff + q, sub, split);
}

template <int TB, int TK>
KernelFn select_kernel(int mode)
{
    if constexpr (TB == TK) {
        if (mode == MODE_DIAG) return eri_class_kernel<TB, TK, MODE_DIAG>;
    }
    return mode == MODE_PACKED ? eri_class_kernel<TB, TK, MODE_PACKED> : nullptr;
}

}  // namespace hfgpu
