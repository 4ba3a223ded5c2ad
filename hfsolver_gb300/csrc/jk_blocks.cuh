// Fock two-electron term G = J - K/2 from the class-wise quartet blocks that
// the ERI kernels leave in HBM (EriArgs::blocks).
//
// Same G as formG (src/scf.f90:26-58) and as jk_packed_kernel, but only the
// quartets that survived Schwarz screening are read (no zeros), reads are
// coalesced (block element e of quartet q is at e * nq + q), and each thread
// folds its whole quartet block into J/K partial sums before the atomics.
//
// Degeneracy: a block holds every component quartet of the shell quartet,
// including both orders when A == B, C == D or bra pair == ket pair; weighting
// every element by 1/2 per coincidence of shells makes the sum over the block
// equal to the sum over unique integrals with the usual 8-fold weights.  The
// half-matrix updates are those of jk.cu:
//   Gh[a][b] += 2 w P_cd, Gh[c][d] += 2 w P_ab,
//   Gh[a][c] -= w P_bd/2, Gh[b][c] -= w P_ad/2, Gh[a][d] -= w P_bc/2, Gh[b][d] -= w P_ac/2,
// and G = Gh + Gh^T.
#pragma once
#include "eri_kernel.cuh"

namespace hfgpu {

struct DigestArgs {
    ShellDev sh;
    PairDev pr;
    const int* gpairs;
    const int64_t* prefix;
    const int2* list;
    const Seg* segs;
    int nseg;
    int64_t nq;
    const double* blocks;
    const double* P;
    int n;
    double* Gh;
    int split;   // lanes per quartet (digest_wide_kernel; a power of two <= 32)
    int rounds;  // a warp screens rounds x (32 / split) quartets and digests the survivors (1 to 8)
    // density-difference screening (screen > 0): pair Schwarz bounds Q and the
    // largest |P| element of each shell pair, Dm[S1 * ns + S2]
    double screen;
    const double* Q;
    const double* Dm;
    int ns;
    // batched plans (mol_n != null): per molecule its basis size, density,
    // half-matrix output, screen (< 0: not part of this build), shell-pair
    // maximum table, shell count and first shell; the scalars above are unused
    const int* mol_n;
    const double* const* mol_P;
    double* const* mol_Gh;
    const double* mol_screen;
    const double* const* mol_Dm;
    const int* mol_ns;
    const int* mol_sh0;
    // the (bra, ket) pair ids of every quartet of the class, written by the ERI
    // pass (null: found by searching the segments), and in batched plans the
    // molecule of every pair
    const int2* qlist;
    const int* pair_mol;
};

// the per-molecule view of a batched build (the arguments themselves for one molecule)
struct DigestMol {
    int n, ns, sh0;
    const double* P;
    double* Gh;
    double screen;
    const double* Dm;
};

__device__ __forceinline__ bool digest_mol(const DigestArgs& a, int mol, DigestMol& m)
{
    if (!a.mol_n) {
        m = DigestMol{a.n, a.ns, 0, a.P, a.Gh, a.screen, a.Dm};
        return true;
    }
    m.screen = a.mol_screen[mol];
    if (m.screen < 0.0) return false;
    m.n = a.mol_n[mol];
    m.ns = a.mol_ns[mol];
    m.sh0 = a.mol_sh0[mol];
    m.P = a.mol_P[mol];
    m.Gh = a.mol_Gh[mol];
    m.Dm = a.mol_Dm ? a.mol_Dm[mol] : nullptr;
    return true;
}

// quartet qg of the class: its bra and ket pair ids and its molecule, from the
// list the ERI pass wrote, else by searching the segments and prefix sums
__device__ __forceinline__ void digest_quartet(const DigestArgs& a, int64_t qg, int& bra, int& ket, int& mol)
{
    if (a.qlist) {
        const int2 e = __ldg(a.qlist + qg);
        bra = e.x;
        ket = e.y;
        mol = a.pair_mol ? __ldg(a.pair_mol + bra) : 0;
        return;
    }
    const int qg32 = (int)qg;
    int lo = 0, hi = a.nseg - 1;  // last segment with qoff <= qg
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((int)(a.segs[mid].qoff) <= qg32) lo = mid; else hi = mid - 1;
    }
    const Seg sg = a.segs[lo];
    const int q = qg32 - (int)sg.qoff;  // class quartet counts stay below 2^31 (plan check)
    mol = sg.mol;
    if (sg.list) {
        const int2 e = a.list[sg.pref0 + q];
        bra = e.x;
        ket = e.y;
        return;
    }
    const int64_t* pf = a.prefix + sg.pref0;
    int l2 = 0, h2 = sg.nbra - 1;
    while (l2 < h2) {
        const int mid = (l2 + h2 + 1) >> 1;
        if ((int)pf[mid] <= q) l2 = mid; else h2 = mid - 1;
    }
    bra = a.gpairs[sg.bra0 + l2];
    ket = a.gpairs[sg.ket0 + (q - (int)pf[l2])];
}

// true if the quartet's whole contribution is below the screening threshold:
// |(ab|cd)| <= Q_bra Q_ket, and the largest density factor it meets is
// 2|P_ab|, 2|P_cd| (Coulomb) or |P_ac|/2 ... (exchange)
__device__ __forceinline__ bool digest_skip(const DigestArgs& a, const DigestMol& m, int bra, int ket, int A, int B,
                                            int C, int D)
{
    if (m.screen <= 0.0) return false;
    const double* Dm = m.Dm;
    const int ns = m.ns;
    A -= m.sh0; B -= m.sh0; C -= m.sh0; D -= m.sh0;
    const double dj = fmax(Dm[A * ns + B], Dm[C * ns + D]);
    const double dk = fmax(fmax(Dm[A * ns + C], Dm[B * ns + D]), fmax(Dm[A * ns + D], Dm[B * ns + C]));
    return a.Q[bra] * a.Q[ket] * fmax(2.0 * dj, 0.5 * dk) < m.screen;
}

// v != 0 tested on the bit pattern (integer pipe; -0 counts as zero)
__device__ __forceinline__ bool digest_nonzero(double v) { return (__double_as_longlong(v) << 1) != 0; }

constexpr int DIGEST_MAX_Q = 256;  // quartets screened per warp: 32 x 8 rounds
// threads per block of the digest kernels (two warps: a class with few quartets
// still reaches most SMs)
constexpr int DIGEST_BLOCK = 64, DIGEST_WARPS = DIGEST_BLOCK / 32;

// Screen the warp's quartets q0 .. q0 + cnt - 1 (density-difference screen,
// molecules not in this build) and leave the offsets of the survivors in the
// warp's list; returns their number.  The survivors are then digested in full
// warps, instead of each warp idling on the lanes whose quartets were skipped.
__device__ __forceinline__ int digest_compact(const DigestArgs& a, int64_t q0, int cnt, int* list, int lane)
{
    int ns = 0;
    for (int r = 0; r < cnt; r += 32) {
        const int k = r + lane;
        const int64_t qg = q0 + k;
        bool keep = false;
        if (k < cnt && qg < a.nq) {
            int bra, ket, mol;
            digest_quartet(a, qg, bra, ket, mol);
            DigestMol mm;
            if (digest_mol(a, mol, mm))
                keep = !digest_skip(a, mm, bra, ket, a.pr.A[bra], a.pr.B[bra], a.pr.A[ket], a.pr.B[ket]);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) list[ns + __popc(m & ((1u << lane) - 1u))] = k;
        ns += __popc(m);
    }
    __syncwarp();
    return ns;
}

// one thread digests one whole quartet (already screened)
template <int TB, int TK>
__device__ __forceinline__ void digest_one(const DigestArgs& a, int64_t qg)
{
    using CI = ClassInfo<TB, TK>;
    constexpr int NA = ncart(CI::LA), NB = ncart(CI::LB), NC = ncart(CI::LC), ND = ncart(CI::LD);
    int bra, ket, mol;
    digest_quartet(a, qg, bra, ket, mol);
    DigestMol mm;
    digest_mol(a, mol, mm);
    const int A = a.pr.A[bra], B = a.pr.B[bra], C = a.pr.A[ket], D = a.pr.B[ket];
    int fa[NA], fb[NB], fc[NC], fd[ND];
#pragma unroll
    for (int i = 0; i < NA; ++i) fa[i] = a.sh.comp_fn[a.sh.cfn0[A] + i];
#pragma unroll
    for (int i = 0; i < NB; ++i) fb[i] = a.sh.comp_fn[a.sh.cfn0[B] + i];
#pragma unroll
    for (int i = 0; i < NC; ++i) fc[i] = a.sh.comp_fn[a.sh.cfn0[C] + i];
#pragma unroll
    for (int i = 0; i < ND; ++i) fd[i] = a.sh.comp_fn[a.sh.cfn0[D] + i];
    const int n = mm.n;
    const double* Pm = mm.P;
    auto Pv = [&](int x, int y) { return (x < 0 || y < 0) ? 0.0 : __ldg(Pm + x + (int64_t)y * n); };
    const double f = (A == B ? 0.5 : 1.0) * (C == D ? 0.5 : 1.0) * (bra == ket ? 0.5 : 1.0);
    // every output is multiplied once by its weight (J: 2f, K: -f/2) instead of
    // every integral by f: on this GPU each FP64 instruction is as dear as an FMA
    const double cj = 2.0 * f, ck = -0.5 * f;
    // accumulators indexed by the rolled (a, b) loop live in local memory; each
    // FMA chain starts from the stored partial sum, so no separate FP64 adds
    double jab[NA * NB], kac[NA * NC], kbc[NB * NC], kad[NA * ND], kbd[NB * ND];
    double jcd[NC * ND], Pcd[NC * ND];
#pragma unroll
    for (int i = 0; i < NA * NC; ++i) kac[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NB * NC; ++i) kbc[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NA * ND; ++i) kad[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NB * ND; ++i) kbd[i] = 0.0;
#pragma unroll
    for (int ic = 0; ic < NC; ++ic)
#pragma unroll
        for (int id = 0; id < ND; ++id) {
            jcd[ic * ND + id] = 0.0;
            Pcd[ic * ND + id] = Pv(fc[ic], fd[id]);
        }
#pragma unroll 1
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll 1
        for (int ib = 0; ib < NB; ++ib) {
            const double Pab = Pv(fa[ia], fb[ib]);
            double Pac[NC], Pbc[NC], Pad[ND], Pbd[ND];
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) {
                Pac[ic] = Pv(fa[ia], fc[ic]);
                Pbc[ic] = Pv(fb[ib], fc[ic]);
            }
#pragma unroll
            for (int id = 0; id < ND; ++id) {
                Pad[id] = Pv(fa[ia], fd[id]);
                Pbd[id] = Pv(fb[ib], fd[id]);
            }
            double s_ab = 0.0, s_ad[ND], s_bd[ND];
#pragma unroll
            for (int id = 0; id < ND; ++id) {
                s_ad[id] = kad[ia * ND + id];
                s_bd[id] = kbd[ib * ND + id];
            }
            const double* blk = a.blocks + (int64_t)((ia * NB + ib) * CI::NCDT) * a.nq + qg;
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) {
                double s_ac = kac[ia * NC + ic], s_bc = kbc[ib * NC + ic];
#pragma unroll
                for (int id = 0; id < ND; ++id) {
                    const double v = __ldg(blk + (int64_t)(ic * ND + id) * a.nq);
                    s_ab = fma(v, Pcd[ic * ND + id], s_ab);
                    jcd[ic * ND + id] = fma(v, Pab, jcd[ic * ND + id]);
                    s_ac = fma(v, Pbd[id], s_ac);
                    s_bc = fma(v, Pad[id], s_bc);
                    s_ad[id] = fma(v, Pbc[ic], s_ad[id]);
                    s_bd[id] = fma(v, Pac[ic], s_bd[id]);
                }
                kac[ia * NC + ic] = s_ac;
                kbc[ib * NC + ic] = s_bc;
            }
            jab[ia * NB + ib] = s_ab;
#pragma unroll
            for (int id = 0; id < ND; ++id) {
                kad[ia * ND + id] = s_ad[id];
                kbd[ib * ND + id] = s_bd[id];
            }
        }
    double* Gh = mm.Gh;
    auto add = [&](int x, int y, double v) {
        if (x >= 0 && y >= 0 && digest_nonzero(v)) atomicAdd(Gh + x + (int64_t)y * n, v);
    };
#pragma unroll 1
    for (int ia = 0; ia < NA; ++ia)
        for (int ib = 0; ib < NB; ++ib) add(fa[ia], fb[ib], cj * jab[ia * NB + ib]);
#pragma unroll 1
    for (int ic = 0; ic < NC; ++ic)
        for (int id = 0; id < ND; ++id) add(fc[ic], fd[id], cj * jcd[ic * ND + id]);
#pragma unroll 1
    for (int ia = 0; ia < NA; ++ia)
        for (int ic = 0; ic < NC; ++ic) add(fa[ia], fc[ic], ck * kac[ia * NC + ic]);
#pragma unroll 1
    for (int ib = 0; ib < NB; ++ib)
        for (int ic = 0; ic < NC; ++ic) add(fb[ib], fc[ic], ck * kbc[ib * NC + ic]);
#pragma unroll 1
    for (int ia = 0; ia < NA; ++ia)
        for (int id = 0; id < ND; ++id) add(fa[ia], fd[id], ck * kad[ia * ND + id]);
#pragma unroll 1
    for (int ib = 0; ib < NB; ++ib)
        for (int id = 0; id < ND; ++id) add(fb[ib], fd[id], ck * kbd[ib * ND + id]);
}

template <int TB, int TK>
__global__ void __launch_bounds__(DIGEST_BLOCK) digest_kernel(DigestArgs a)
{
    __shared__ int sl[DIGEST_WARPS][DIGEST_MAX_Q];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int qpw = 32 * a.rounds;
    const int64_t q0 = ((int64_t)blockIdx.x * DIGEST_WARPS + warp) * qpw;
    if (q0 >= a.nq) return;  // the whole warp
    if (a.screen <= 0.0 && !a.mol_n) {  // nothing is screened: no list
        for (int k = lane; k < qpw; k += 32)
            if (q0 + k < a.nq) digest_one<TB, TK>(a, q0 + k);
        return;
    }
    const int ns = digest_compact(a, q0, qpw, sl[warp], lane);
    for (int base = 0; base < ns; base += 32)
        if (base + lane < ns) digest_one<TB, TK>(a, q0 + sl[warp][base + lane]);
}

// The same Fock contribution with `split` lanes per quartet, for classes with
// few quartets and large blocks ((dd|dd) has a few hundred quartets of 1296
// elements each): the lanes of a quartet take its (a, b) rows in turn, send
// each row's J_ab and K contributions straight to Gh, and sum their partial
// J_cd with warp shuffles before one lane per (c, d) adds it.
template <int TB, int TK>
__device__ __forceinline__ void digest_wide_one(const DigestArgs& a, int64_t qg, int split, int sub, unsigned mask)
{
    using CI = ClassInfo<TB, TK>;
    constexpr int NA = ncart(CI::LA), NB = ncart(CI::LB), NC = ncart(CI::LC), ND = ncart(CI::LD);
    int bra, ket, mol;
    digest_quartet(a, qg, bra, ket, mol);
    DigestMol mm;
    digest_mol(a, mol, mm);
    const int A = a.pr.A[bra], B = a.pr.B[bra], C = a.pr.A[ket], D = a.pr.B[ket];
    int fc[NC], fd[ND];
#pragma unroll
    for (int i = 0; i < NC; ++i) fc[i] = a.sh.comp_fn[a.sh.cfn0[C] + i];
#pragma unroll
    for (int i = 0; i < ND; ++i) fd[i] = a.sh.comp_fn[a.sh.cfn0[D] + i];
    const int* fa = a.sh.comp_fn + a.sh.cfn0[A];
    const int* fb = a.sh.comp_fn + a.sh.cfn0[B];
    const int n = mm.n;
    const double* Pm = mm.P;
    auto Pv = [&](int x, int y) { return (x < 0 || y < 0) ? 0.0 : __ldg(Pm + x + (int64_t)y * n); };
    double* Gh = mm.Gh;
    auto add = [&](int x, int y, double v) {
        if (x >= 0 && y >= 0 && digest_nonzero(v)) atomicAdd(Gh + x + (int64_t)y * n, v);
    };
    const double f = (A == B ? 0.5 : 1.0) * (C == D ? 0.5 : 1.0) * (bra == ket ? 0.5 : 1.0);
    const double cj = 2.0 * f, ck = -0.5 * f;
    double jcd[NC * ND], Pcd[NC * ND];
#pragma unroll
    for (int ic = 0; ic < NC; ++ic)
#pragma unroll
        for (int id = 0; id < ND; ++id) {
            jcd[ic * ND + id] = 0.0;
            Pcd[ic * ND + id] = Pv(fc[ic], fd[id]);
        }
#pragma unroll 1
    for (int ab = sub; ab < NA * NB; ab += split) {
        const int ia = ab / NB, ib = ab - ia * NB;
        const int xa = __ldg(fa + ia), xb = __ldg(fb + ib);
        const double Pab = Pv(xa, xb);
        double Pac[NC], Pbc[NC], Pad[ND], Pbd[ND];
#pragma unroll
        for (int ic = 0; ic < NC; ++ic) {
            Pac[ic] = Pv(xa, fc[ic]);
            Pbc[ic] = Pv(xb, fc[ic]);
        }
#pragma unroll
        for (int id = 0; id < ND; ++id) {
            Pad[id] = Pv(xa, fd[id]);
            Pbd[id] = Pv(xb, fd[id]);
        }
        double s_ab = 0.0, s_ad[ND], s_bd[ND];
#pragma unroll
        for (int id = 0; id < ND; ++id) s_ad[id] = s_bd[id] = 0.0;
        const double* blk = a.blocks + (int64_t)(ab * CI::NCDT) * a.nq + qg;
#pragma unroll
        for (int ic = 0; ic < NC; ++ic) {
            double s_ac = 0.0, s_bc = 0.0;
#pragma unroll
            for (int id = 0; id < ND; ++id) {
                const double v = __ldg(blk + (int64_t)(ic * ND + id) * a.nq);
                s_ab = fma(v, Pcd[ic * ND + id], s_ab);
                jcd[ic * ND + id] = fma(v, Pab, jcd[ic * ND + id]);
                s_ac = fma(v, Pbd[id], s_ac);
                s_bc = fma(v, Pad[id], s_bc);
                s_ad[id] = fma(v, Pbc[ic], s_ad[id]);
                s_bd[id] = fma(v, Pac[ic], s_bd[id]);
            }
            add(xa, fc[ic], ck * s_ac);
            add(xb, fc[ic], ck * s_bc);
        }
        add(xa, xb, cj * s_ab);
#pragma unroll
        for (int id = 0; id < ND; ++id) {
            add(xa, fd[id], ck * s_ad[id]);
            add(xb, fd[id], ck * s_bd[id]);
        }
    }
    for (int o = split >> 1; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < NC * ND; ++i) jcd[i] += __shfl_xor_sync(mask, jcd[i], o);
#pragma unroll
    for (int i = 0; i < NC * ND; ++i)
        if ((i & (split - 1)) == sub) add(fc[i / ND], fd[i % ND], cj * jcd[i]);
}

template <int TB, int TK>
__global__ void __launch_bounds__(DIGEST_BLOCK) digest_wide_kernel(DigestArgs a)
{
    __shared__ int sl[DIGEST_WARPS][DIGEST_MAX_Q];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int split = a.split, per = 32 / split;
    const int qpw = per * a.rounds;
    const int64_t q0 = ((int64_t)blockIdx.x * DIGEST_WARPS + warp) * qpw;
    if (q0 >= a.nq) return;  // the whole warp
    const int sub = lane & (split - 1);
    const unsigned mask = split == 32 ? 0xffffffffu : (((1u << split) - 1u) << (lane & ~(unsigned)(split - 1)));
    if (a.screen <= 0.0 && !a.mol_n) {  // nothing is screened: no list
        for (int base = 0; base < qpw; base += per) {
            const int64_t qg = q0 + base + lane / split;  // the same for all lanes of a quartet
            if (qg < a.nq) digest_wide_one<TB, TK>(a, qg, split, sub, mask);
        }
        return;
    }
    const int ns = digest_compact(a, q0, qpw, sl[warp], lane);
    for (int base = 0; base < ns; base += per) {
        const int k = base + lane / split;  // the same for all lanes of a quartet
        if (k < ns) digest_wide_one<TB, TK>(a, q0 + sl[warp][k], split, sub, mask);
    }
}

using DigestFn = void (*)(DigestArgs);
DigestFn digest_fn(int tb, int tk);       // jk_blocks.cu
DigestFn digest_wide_fn(int tb, int tk);  // jk_blocks.cu

}  // namespace hfgpu
