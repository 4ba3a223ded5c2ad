// Contracted electron-repulsion integrals (ab|cd) in FP64 on sm_103a.
//
// Replaces hfsolver's getInts -> contr_coulomb -> coulomb_repulsion
// (src/qc.c:95-131, src/cints.c:72-183): the same contracted Cartesian
// integrals, written into the same 8-fold packed array, but evaluated
// shell-quartet-at-a-time with the McMurchie-Davidson scheme instead of one
// Cartesian primitive quartet at a time with the THO formula.
//
//   (ab|cd) = 2 pi^{5/2} / (p q sqrt(p+q)) sum_{tuv} E^{ab}_{tuv}
//             sum_{t'u'v'} (-1)^{t'+u'+v'} E^{cd}_{t'u'v'} R_{t+t',u+u',v+v'}(alpha, P-Q)
//
// GB300 layout and mapping:
//  * Primitive-pair records (p, P and the Hermite coefficients of every
//    component pair, scaled by the contraction coefficients, exp(-mu R_AB^2)
//    and 1/p) are built once per molecule by pair_data_kernel and stay in HBM
//    (L2-resident for molecules of a few hundred functions).
//  * Quartets are grouped by class (bra pair type <= ket pair type, six pair
//    types ss..dd) and by primitive count, so every warp runs a uniform loop.
//    Each class is one kernel instantiation whose component loops are fully
//    unrolled at compile time: only the non-zero Hermite terms are touched.
//  * The ket's Cartesian components are split into G chunks of NCD; a warp
//    handles 32 quartets for one chunk (warp-uniform), so each thread keeps
//    NAB x NCD accumulators in registers.
//  * Schwarz screening: pairs of a group are sorted by decreasing bound
//    Q = sqrt(max |(ab|ab)|), so the kets surviving Q_bra Q_ket >= thr form a
//    prefix; quartets are enumerated from prefix sums (no quartet list).
#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>

#include "boys.cuh"
#include "eri_kernel.cuh"
#include "internal.h"
#include "autotune.h"
#include "eri_plan.h"
#include "jk_blocks.cuh"
#include "md.cuh"

namespace hfgpu {

int64_t packed_size(int64_t n)
{
    int64_t m = n * (n + 1) / 2;
    return m * (m + 1) / 2;
}

__host__ __device__ __forceinline__ int64_t packed_index(int64_t i, int64_t j, int64_t k, int64_t l)
{
    int64_t a = i > j ? i : j, b = i > j ? j : i;
    int64_t c = k > l ? k : l, d = k > l ? l : k;
    int64_t ij = a * (a + 1) / 2 + b, kl = c * (c + 1) / 2 + d;
    return ij >= kl ? ij * (ij + 1) / 2 + kl : kl * (kl + 1) / 2 + ij;
}

// ------------------------------------------------------------------ pair data
template <int LA, int LB>
__device__ __forceinline__ void hermite_1d(double (&E)[LA + 1][LB + 1][LA + LB + 1], double xpa, double xpb,
                                           double i2p)
{
#pragma unroll
    for (int i = 0; i <= LA; ++i)
#pragma unroll
        for (int j = 0; j <= LB; ++j)
#pragma unroll
            for (int t = 0; t <= LA + LB; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
#pragma unroll
    for (int i = 0; i < LA; ++i)
#pragma unroll
        for (int t = 0; t <= i + 1; ++t) {
            double v = xpa * E[i][0][t];
            if (t > 0) v = fma(i2p, E[i][0][t - 1], v);
            if (t + 1 <= i) v = fma((double)(t + 1), E[i][0][t + 1], v);
            E[i + 1][0][t] = v;
        }
#pragma unroll
    for (int i = 0; i <= LA; ++i)
#pragma unroll
        for (int j = 0; j < LB; ++j)
#pragma unroll
            for (int t = 0; t <= i + j + 1; ++t) {
                double v = xpb * E[i][j][t];
                if (t > 0) v = fma(i2p, E[i][j][t - 1], v);
                if (t + 1 <= i + j) v = fma((double)(t + 1), E[i][j][t + 1], v);
                E[i][j + 1][t] = v;
            }
}

template <int T>
__global__ void pair_data_kernel(ShellDev sh, PairDev pr, const int4* items, int nitems, double* pdata)
{
    constexpr int LA = ptype_la(T), LB = ptype_lb(T);
    constexpr int STRIDE = pair_stride(LA, LB);
    int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nitems) return;
    int4 item = items[it];
    int P = item.x, ia = item.y, ib = item.z;
    int A = pr.A[P], B = pr.B[P];
    double a = sh.alpha[sh.prim0[A] + ia], b = sh.alpha[sh.prim0[B] + ib];
    double ax = sh.xyz[3 * A], ay = sh.xyz[3 * A + 1], az = sh.xyz[3 * A + 2];
    double bx = sh.xyz[3 * B], by = sh.xyz[3 * B + 1], bz = sh.xyz[3 * B + 2];
    double p = a + b, ip = 1.0 / p, mu = a * b * ip;
    double px = (a * ax + b * bx) * ip, py = (a * ay + b * by) * ip, pz = (a * az + b * bz) * ip;
    double rab2 = (ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz);
    double kab = exp(-mu * rab2) * ip;
    double Ex[LA + 1][LB + 1][LA + LB + 1], Ey[LA + 1][LB + 1][LA + LB + 1], Ez[LA + 1][LB + 1][LA + LB + 1];
    hermite_1d<LA, LB>(Ex, px - ax, px - bx, 0.5 * ip);
    hermite_1d<LA, LB>(Ey, py - ay, py - by, 0.5 * ip);
    hermite_1d<LA, LB>(Ez, pz - az, pz - bz, 0.5 * ip);
    int nb = sh.nprim[B];
    double* rec = pdata + pr.off[P] + (int64_t)(ia * nb + ib) * STRIDE;
    rec[0] = p;
    rec[1] = px;
    rec[2] = py;
    rec[3] = pz;
    const double* ca = sh.coef + sh.coef0[A];
    const double* cb = sh.coef + sh.coef0[B];
    int npa = sh.nprim[A];
#pragma unroll
    for (int ca_i = 0; ca_i < ncart(LA); ++ca_i)
#pragma unroll
        for (int cb_i = 0; cb_i < ncart(LB); ++cb_i) {
            const Cart c1 = cart(LA, ca_i), c2 = cart(LB, cb_i);
            double s = ca[ca_i * npa + ia] * cb[cb_i * nb + ib] * kab;
            double* e = rec + PAIR_HDR + eoff(LA, LB, ca_i, cb_i);
            int w = 0;
#pragma unroll
            for (int t = 0; t <= c1.l + c2.l; ++t)
#pragma unroll
                for (int u = 0; u <= c1.m + c2.m; ++u)
#pragma unroll
                    for (int v = 0; v <= c1.n + c2.n; ++v)
                        e[w++] = s * Ex[c1.l][c2.l][t] * Ey[c1.m][c2.m][u] * Ez[c1.n][c2.n][v];
        }
}

// ------------------------------------------------------------------ host side
#define HF_DECL(B, K) KernelFn eri_kernel_##B##K(int mode);
HF_DECL(0, 0) HF_DECL(0, 1) HF_DECL(0, 2) HF_DECL(0, 3) HF_DECL(0, 4) HF_DECL(0, 5)
HF_DECL(1, 1) HF_DECL(1, 2) HF_DECL(1, 3) HF_DECL(1, 4) HF_DECL(1, 5)
HF_DECL(2, 2) HF_DECL(2, 3) HF_DECL(2, 4) HF_DECL(2, 5)
HF_DECL(3, 3) HF_DECL(3, 4) HF_DECL(3, 5)
HF_DECL(4, 4) HF_DECL(4, 5)
HF_DECL(5, 5)
#undef HF_DECL

static KernelFn get_kernel(int tb, int tk, int mode)
{
    static KernelFn (*const table[6][6])(int) = {
        {eri_kernel_00, eri_kernel_01, eri_kernel_02, eri_kernel_03, eri_kernel_04, eri_kernel_05},
        {nullptr, eri_kernel_11, eri_kernel_12, eri_kernel_13, eri_kernel_14, eri_kernel_15},
        {nullptr, nullptr, eri_kernel_22, eri_kernel_23, eri_kernel_24, eri_kernel_25},
        {nullptr, nullptr, nullptr, eri_kernel_33, eri_kernel_34, eri_kernel_35},
        {nullptr, nullptr, nullptr, nullptr, eri_kernel_44, eri_kernel_45},
        {nullptr, nullptr, nullptr, nullptr, nullptr, eri_kernel_55}};
    KernelFn f = table[tb][tk] ? table[tb][tk](mode) : nullptr;
    HF_CHECK(f != nullptr, HFGPU_ERR_CUDA, "missing ERI kernel for class");
    return f;
}

// event-timed duration of the work between a and b (waits for b)
static float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    HF_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, a, b));
    return ms;
}

// lanes per quartet for kb x kk primitive quartets: enough independent work per
// lane (between target and 2 target primitive quartets) without idling the rest
// of the warp
static int pick_split(int64_t kprod, int target = 16)
{
    int s = 1;
    while (s < 32 && kprod >= 2 * (int64_t)target * s) s <<= 1;
    return s;
}

static int class_G(int tb, int tk)
{
    int nab = ncart(ptype_la(tb)) * ncart(ptype_lb(tb));
    int ncd = ncart(ptype_la(tk)) * ncart(ptype_lb(tk));
    return ncd / pick_ncd(nab, ncd);
}

// McMurchie-Davidson reference flop count of one primitive quartet:
//   30 + 3L + 2 C(L+4,4) + 2 nc_c nc_d nH(Lp) nH(Lq) + 2 nc_a nc_b nc_c nc_d nH(Lp)
double md_flops(int la, int lb, int lc, int ld)
{
    auto binom4 = [](int n) { return (double)n * (n - 1) * (n - 2) * (n - 3) / 24.0; };
    int Lp = la + lb, Lq = lc + ld, L = Lp + Lq;
    return 30 + 3.0 * L + 2 * binom4(L + 4) + 2.0 * ncart(lc) * ncart(ld) * nherm(Lp) * nherm(Lq) +
           2.0 * ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) * nherm(Lp);
}

static void launch_class(Context& ctx, EriPlan* P, ClassPlan& c, int mode, double* out, const int2* list,
                         double* blocks = nullptr, cudaStream_t on = nullptr)
{
    if (c.nwarps == 0) return;
    EriArgs a;
    a.blocks = blocks;
    a.qlist = (blocks && mode == MODE_PACKED && P->qlist.p) ? P->qlist.p + c.qbase : nullptr;
    a.nq_class = c.nq;
    a.mol_out = mode == MODE_PACKED ? P->mol_out.p : nullptr;
    a.sh = P->shdev();
    a.pr = P->prdev();
    a.boys = ctx.boys;
    a.gpairs = P->gpairs.p;
    a.prefix = P->prefix.p;
    a.list = list;
    a.segs = c.dsegs.p;
    a.nseg = (int)c.segs.size();
    a.nwarps = c.nwarps;
    a.out = out;
    const int64_t nblocks = (c.nwarps + ERI_BLOCK / 32 - 1) / (ERI_BLOCK / 32);
    get_kernel(c.tb, c.tk, mode)<<<(unsigned)nblocks, ERI_BLOCK, 0, on ? on : ctx.stream>>>(a);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

// Schwarz factor of each shell pair from its diagonal quartet block (36 slots)
__global__ void pair_qmax_kernel(int npair, const double* __restrict__ diag, double* Q)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= npair) return;
    double m = 0.0;
    for (int k = 0; k < 36; ++k) m = fmax(m, fabs(diag[(int64_t)id * 36 + k]));
    Q[id] = sqrt(m);
}

EriPlan* eri_plan_create(Context& ctx, const Basis& b, double thr)
{
    cudaStream_t st = ctx.stream;
    auto P = new EriPlan();
    try {
        P->basis = b;
        const int ns = (int)b.shells.size();
        std::vector<int> L(ns), np(ns), p0(ns), c0(ns), f0(ns);
        std::vector<double> xyz(3 * ns);
        for (int s = 0; s < ns; s++) {
            const Shell& sh = b.shells[s];
            L[s] = sh.L; np[s] = sh.nprim; p0[s] = sh.prim0; c0[s] = sh.coef0; f0[s] = sh.cfn0;
            xyz[3 * s] = sh.x; xyz[3 * s + 1] = sh.y; xyz[3 * s + 2] = sh.z;
        }
        P->sL = to_device(L, st); P->snp = to_device(np, st); P->sp0 = to_device(p0, st);
        P->sc0 = to_device(c0, st); P->scf = to_device(f0, st); P->cfn = to_device(b.comp_fn, st);
        P->sxyz = to_device(xyz, st); P->alpha = to_device(b.alpha, st); P->coef = to_device(b.coef, st);
        ctx.trace_mark("plan shells");

        // shell pairs, larger angular momentum first
        int64_t off = 0;
        std::vector<int4> items[NPTYPE];
        for (int i = 0; i < ns; i++)
            for (int j = 0; j <= i; j++) {
                int A = i, B = j;
                if (L[A] < L[B]) std::swap(A, B);
                int t = ptype_of(L[A], L[B]);
                int id = (int)P->pA.size();
                P->pA.push_back(A); P->pB.push_back(B); P->pT.push_back(t);
                P->pK.push_back(np[A] * np[B]);
                P->poff.push_back(off);
                for (int x = 0; x < np[A]; x++)
                    for (int y = 0; y < np[B]; y++) items[t].push_back(make_int4(id, x, y, 0));
                off += (int64_t)np[A] * np[B] * pair_stride(ptype_la(t), ptype_lb(t));
            }
        P->npair = (int)P->pA.size();
        P->dA = to_device(P->pA, st); P->dB = to_device(P->pB, st); P->dK = to_device(P->pK, st);
        P->doff = to_device(P->poff, st);
        P->pdata.alloc(off, st);
        for (int t = 0; t < NPTYPE; t++) {
            if (items[t].empty()) continue;
            DBuf<int4> di = to_device(items[t], st);
            int n = (int)items[t].size();
            int blocks = (n + 127) / 128;
            ShellDev sd = P->shdev();
            PairDev pd = P->prdev();
            switch (t) {
                case 0: pair_data_kernel<0><<<blocks, 128, 0, st>>>(sd, pd, di.p, n, P->pdata.p); count_launch(); break;
                case 1: pair_data_kernel<1><<<blocks, 128, 0, st>>>(sd, pd, di.p, n, P->pdata.p); count_launch(); break;
                case 2: pair_data_kernel<2><<<blocks, 128, 0, st>>>(sd, pd, di.p, n, P->pdata.p); count_launch(); break;
                case 3: pair_data_kernel<3><<<blocks, 128, 0, st>>>(sd, pd, di.p, n, P->pdata.p); count_launch(); break;
                case 4: pair_data_kernel<4><<<blocks, 128, 0, st>>>(sd, pd, di.p, n, P->pdata.p); count_launch(); break;
                case 5: pair_data_kernel<5><<<blocks, 128, 0, st>>>(sd, pd, di.p, n, P->pdata.p); count_launch(); break;
            }
            HF_CUDA(cudaGetLastError());
        }

        ctx.trace_mark("plan pair data");
        // groups: (pair type, primitive count)
        std::map<std::pair<int, int>, std::vector<int>> gmap;
        for (int id = 0; id < P->npair; id++) gmap[{P->pT[id], P->pK[id]}].push_back(id);

        // Schwarz bounds from the diagonal quartets (ab|ab)
        P->Q.assign(P->npair, 1.0);
        if (thr > 0) {
            std::vector<int2> dl;
            std::vector<ClassPlan> dcls;
            for (auto& g : gmap) {
                int t = g.first.first;
                ClassPlan c;
                c.tb = t; c.tk = t;
                Seg s{};
                s.warp0 = 0; s.nq = (int64_t)g.second.size(); s.pref0 = (int64_t)dl.size();
                s.list = 1;
                s.qoff = 0;
                s.split = pick_split((int64_t)g.first.second * g.first.second);
                const int64_t qpw = 32 / s.split;
                for (int id : g.second) dl.push_back(make_int2(id, id));
                bool merged = false;
                for (auto& dc : dcls)
                    if (dc.tb == t) {
                        s.warp0 = dc.nwarps;
                        dc.segs.push_back(s);
                        dc.nwarps += (s.nq + qpw - 1) / qpw * class_G(t, t);
                        merged = true;
                    }
                if (!merged) {
                    c.segs.push_back(s);
                    c.nwarps = (s.nq + qpw - 1) / qpw * class_G(t, t);
                    dcls.push_back(std::move(c));
                }
            }
            DBuf<int2> ddl = to_device(dl, st);
            DBuf<double> diag((size_t)P->npair * 36, st);
            diag.zero();
            for (auto& c : dcls) c.dsegs = to_device(c.segs, st);
            // one small class per pair type, each latency-bound: side by side
            ctx.fork();
            for (size_t i = 0; i < dcls.size(); ++i)
                launch_class(ctx, P, dcls[i], MODE_DIAG, diag.p, ddl.p, nullptr, ctx.aux[i % Context::NAUX]);
            ctx.join();
            // Q = sqrt(max |(ab|ab)|) per pair on the device; only Q comes back
            DBuf<double> dq(P->npair, st);
            pair_qmax_kernel<<<(P->npair + 127) / 128, 128, 0, st>>>(P->npair, diag.p, dq.p);
            count_launch();
            HF_CUDA(cudaGetLastError());
            dq.download(P->Q.data(), P->npair);
            HF_CUDA(cudaStreamSynchronize(st));
            for (auto& g : gmap)
                std::stable_sort(g.second.begin(), g.second.end(),
                                 [&](int x, int y) { return P->Q[x] > P->Q[y]; });
        }

        ctx.trace_mark("plan schwarz");
        // flatten the groups
        std::vector<int> gp;
        struct G { int t, k, off, n; std::vector<double> q; std::vector<int64_t> eff; };
        std::vector<G> groups;
        for (auto& g : gmap) {
            G gg{g.first.first, g.first.second, (int)gp.size(), (int)g.second.size(), {}, {}};
            gg.eff.push_back(0);
            for (int id : g.second) {
                gp.push_back(id);
                gg.q.push_back(P->Q[id]);
                int A = P->pA[id], B = P->pB[id];
                int64_t na = 0, nb = 0;
                for (int c = 0; c < ncart(L[A]); c++) na += b.comp_fn[f0[A] + c] >= 0;
                for (int c = 0; c < ncart(L[B]); c++) nb += b.comp_fn[f0[B] + c] >= 0;
                int64_t e = (A == B) ? na * (na + 1) / 2 : na * nb;
                gg.eff.push_back(gg.eff.back() + e);
            }
            groups.push_back(std::move(gg));
        }
        P->gpairs = to_device(gp, st);
        P->h_gpairs = gp;
        P->dQ = to_device(P->Q, st);

        // segments per class
        std::vector<int64_t> prefix;
        EriStats stt;
        for (int tb = 0; tb < NPTYPE; tb++)
            for (int tk = tb; tk < NPTYPE; tk++) {
                ClassPlan c;
                c.tb = tb; c.tk = tk;
                int G_ = class_G(tb, tk);
                double fl = md_flops(ptype_la(tb), ptype_lb(tb), ptype_la(tk), ptype_lb(tk));
                for (size_t g1 = 0; g1 < groups.size(); g1++) {
                    if (groups[g1].t != tb) continue;
                    for (size_t g2 = 0; g2 < groups.size(); g2++) {
                        if (groups[g2].t != tk) continue;
                        if (tb == tk && g2 < g1) continue;
                        const G& A_ = groups[g1];
                        const G& B_ = groups[g2];
                        bool same = g1 == g2;
                        Seg s{};
                        s.pref0 = (int64_t)prefix.size();
                        s.bra0 = A_.off; s.ket0 = B_.off; s.nbra = A_.n; s.list = 0;
                        int64_t acc = 0, nbf = 0;
                        prefix.push_back(0);
                        for (int i = 0; i < A_.n; i++) {
                            int64_t cnt;
                            if (thr > 0) {
                                double need = A_.q[i] > 0 ? thr / A_.q[i] : INFINITY;
                                // number of leading kets with q >= need (q sorted descending)
                                cnt = std::upper_bound(B_.q.begin(), B_.q.end(), need,
                                                       [](double v, double e) { return v > e; }) -
                                      B_.q.begin();
                            } else {
                                cnt = B_.n;
                            }
                            if (same) cnt = std::min<int64_t>(cnt, i + 1);
                            acc += cnt;
                            prefix.push_back(acc);
                            int64_t ei = A_.eff[i + 1] - A_.eff[i];
                            int64_t sum = B_.eff[cnt];
                            nbf += ei * sum;
                            if (same && cnt == i + 1) nbf -= ei * ei - ei * (ei + 1) / 2;
                        }
                        if (acc == 0) {
                            prefix.resize(s.pref0);
                            continue;
                        }
                        s.nq = acc;
                        s.warp0 = c.nwarps;
                        s.qoff = c.nq;
                        s.split = pick_split((int64_t)A_.k * B_.k);
                        c.kprod.push_back((int64_t)A_.k * B_.k);
                        const int64_t qpw = 32 / s.split;
                        c.nq += acc;
                        c.nwarps += (acc + qpw - 1) / qpw * G_;
                        c.segs.push_back(s);
                        stt.n_quartets += acc;
                        stt.n_bf_quartets += nbf;
                        stt.n_prim_quartets += acc * A_.k * B_.k;
                        stt.flops += (double)acc * A_.k * B_.k * fl;
                    }
                }
                if (!c.segs.empty()) {
                    // the kernels index quartets, warps and prefix sums of a class in 32 bits
                    HF_CHECK(c.nq < (1ll << 31) && c.nwarps < (1ll << 30), HFGPU_ERR_UNSUPPORTED,
                             "quartet class too large for 32-bit indexing");
                    c.dsegs = to_device(c.segs, st);
                    P->classes.push_back(std::move(c));
                }
            }
        P->prefix = to_device(prefix, st);
        P->h_prefix = prefix;
        P->nmol = 1;
        P->mol_nbf = {b.nbf};
        P->mol_ns = {ns};
        P->mol_sh0 = {0};
        P->stats = stt;
        HF_CUDA(cudaStreamSynchronize(st));
        ctx.trace_mark("plan classes");
        return P;
    } catch (...) {
        delete P;
        throw;
    }
}

void eri_plan_destroy(EriPlan* p) { delete p; }

__global__ void sym_kernel(int n, const double* __restrict__ Gh, double* G)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    const int i = idx % n, j = idx / n;
    G[idx] = Gh[idx] + Gh[j + (int64_t)i * n];
}

// lanes per quartet in the Fock digest: spread a class with few quartets and
// large blocks over more lanes (at most one (a, b) row each), up to about
// 150k threads in flight
static int digest_split(const ClassPlan& c)
{
    const int nab = ncart(ptype_la(c.tb)) * ncart(ptype_lb(c.tb));
    int s = 1;
    while (s * 2 <= 32 && s * 2 <= nab && c.nq * s < 150000) s *= 2;
    return s;
}

// largest |P| element of each shell pair
__global__ void shell_dmax_kernel(int ns, const int* __restrict__ L, const int* __restrict__ cfn0,
                                  const int* __restrict__ comp_fn, const double* __restrict__ P, int n,
                                  double* __restrict__ Dm)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ns * ns) return;
    const int s1 = idx / ns, s2 = idx - s1 * ns;
    const int n1 = ncart(L[s1]), n2 = ncart(L[s2]);
    double m = 0.0;
    for (int i = 0; i < n1; ++i) {
        const int f = comp_fn[cfn0[s1] + i];
        if (f < 0) continue;
        for (int j = 0; j < n2; ++j) {
            const int g = comp_fn[cfn0[s2] + j];
            if (g >= 0) m = fmax(m, fabs(P[f + (int64_t)g * n]));
        }
    }
    Dm[idx] = m;
}

// quartets a warp screens before digesting the survivors: one pass when nothing
// is screened; with a screen, up to 8 passes as long as the class still has
// about 16 warps per SM
static int digest_rounds(const Context& ctx, const ClassPlan& c, int split, bool screened)
{
    if (!screened) return 1;
    const int64_t warps1 = (c.nq * split + 31) / 32;
    int r = 1;
    while (r < 8 && warps1 / (2 * r) >= (int64_t)ctx.num_sms * 16) r *= 2;
    return r;
}

static void launch_digest(const ClassPlan& c, const DigestArgs& a, cudaStream_t s)
{
    const int64_t qpw = (int64_t)(32 / a.split) * a.rounds;
    const int64_t warps = (c.nq + qpw - 1) / qpw;
    const unsigned blocks = (unsigned)((warps + DIGEST_WARPS - 1) / DIGEST_WARPS);
    if (a.split == 1)
        digest_fn(c.tb, c.tk)<<<blocks, DIGEST_BLOCK, 0, s>>>(a);
    else
        digest_wide_fn(c.tb, c.tk)<<<blocks, DIGEST_BLOCK, 0, s>>>(a);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

// Lanes per quartet of the class's Fock digest: the built-in rule, or with
// tuning on the fastest of 1, 2, 4, ... lanes timed once per (class, size
// bucket) into a scratch matrix.
static int digest_split_tuned(Context& ctx, const ClassPlan& c, DigestArgs a, int64_t nn)
{
    int split = digest_split(c);
    if (!ctx.tune || c.nq == 0) return split;
    const int bucket = tune_bucket(c.nq);
    if (tune_get(TUNE_DIGEST, c.tb, c.tk, bucket, &split)) return split;
    const int nab = ncart(ptype_la(c.tb)) * ncart(ptype_lb(c.tb));
    DBuf<double> scratch(nn, ctx.stream);
    scratch.zero();
    a.Gh = scratch.p;
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int cand = 1; cand <= 32 && (cand == 1 || cand / 2 < nab); cand <<= 1) {
        a.split = cand;
        a.rounds = digest_rounds(ctx, c, cand, a.screen > 0);
        HF_CUDA(cudaEventRecord(e0, ctx.stream));
        launch_digest(c, a, ctx.stream);
        HF_CUDA(cudaEventRecord(e1, ctx.stream));
        const float ms = elapsed(e0, e1);
        if (ms < best) {
            best = ms;
            split = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tune_set(TUNE_DIGEST, c.tb, c.tk, bucket, split);
    return split;
}

void eri_digest(Context& ctx, EriPlan* P, const double* dP, double* dG, double screen)
{
    HF_CHECK(P->blocks.p != nullptr, HFGPU_ERR_INVALID, "eri_digest: integrals were not kept");
    const int n = P->basis.nbf;
    const int64_t nn = (int64_t)n * n;
    DBuf<double> Gh(nn, ctx.stream);
    Gh.zero();
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    HF_CUDA(cudaEventRecord(e0, ctx.stream));
    const int ns = (int)P->basis.shells.size();
    DBuf<double> Dm;
    if (screen > 0) {
        Dm.alloc((size_t)ns * ns, ctx.stream);
        shell_dmax_kernel<<<(ns * ns + 127) / 128, 128, 0, ctx.stream>>>(ns, P->sL.p, P->scf.p, P->cfn.p, dP, n,
                                                                        Dm.p);
        count_launch();
        HF_CUDA(cudaGetLastError());
    }
    // the classes are independent until the symmetrisation: spread them over the
    // side streams, largest blocks first
    ctx.fork();
    int slot = 0;
    for (int ci = (int)P->classes.size() - 1; ci >= 0; --ci) {
        auto& c = P->classes[ci];
        if (c.nq == 0) continue;
        DigestArgs a;
        a.sh = P->shdev();
        a.pr = P->prdev();
        a.gpairs = P->gpairs.p;
        a.prefix = P->prefix.p;
        a.list = nullptr;
        a.segs = c.dsegs.p;
        a.nseg = (int)c.segs.size();
        a.nq = c.nq;
        a.blocks = P->blocks.p + c.boff;
        a.P = dP;
        a.n = n;
        a.Gh = Gh.p;
        a.screen = screen;
        a.Q = P->dQ.p;
        a.Dm = Dm.p;
        a.ns = ns;
        a.mol_n = nullptr;
        a.mol_P = nullptr;
        a.mol_Gh = nullptr;
        a.mol_screen = nullptr;
        a.mol_Dm = nullptr;
        a.mol_ns = nullptr;
        a.mol_sh0 = nullptr;
        a.qlist = P->qlist.p ? P->qlist.p + c.qbase : nullptr;
        a.pair_mol = nullptr;
        a.rounds = 1;
        a.split = digest_split_tuned(ctx, c, a, nn);
        a.rounds = digest_rounds(ctx, c, a.split, screen > 0);
        cudaStream_t s = ctx.aux[slot++ % Context::NAUX];
        launch_digest(c, a, s);
    }
    ctx.join();
    sym_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, ctx.stream>>>(n, Gh.p, dG);
    count_launch();
    HF_CUDA(cudaGetLastError());
    HF_CUDA(cudaEventRecord(e1, ctx.stream));
    ctx.fock_events.push_back({e0, e1, screen <= 0});  // timed later, without a host wait here
}
EriStats eri_plan_stats(const EriPlan* p) { return p->stats; }

void eri_compute_packed(Context& ctx, EriPlan* P, double* d_out, EriStats* st)
{
    eri_compute(ctx, P, d_out, false, st);
}

static int block_size(int tb, int tk)
{
    return ncart(ptype_la(tb)) * ncart(ptype_lb(tb)) * ncart(ptype_la(tk)) * ncart(ptype_lb(tk));
}

// lay the warps of a class out again for another lanes-per-quartet target
static void layout_class(Context& ctx, ClassPlan& c, int target)
{
    const int G_ = class_G(c.tb, c.tk);
    c.nwarps = 0;
    for (size_t i = 0; i < c.segs.size(); ++i) {
        Seg& s = c.segs[i];
        s.split = pick_split(c.kprod[i], target);
        s.warp0 = c.nwarps;
        const int64_t qpw = 32 / s.split;
        c.nwarps += (s.nq + qpw - 1) / qpw * G_;
    }
    HF_CHECK(c.nwarps < (1ll << 30), HFGPU_ERR_UNSUPPORTED, "quartet class too large for 32-bit indexing");
    c.dsegs.upload(c.segs.data(), c.segs.size());
    c.lane_target = target;
}

// The ERI launch of a class with the tuned lanes-per-quartet target.  On the
// first molecule of a (class, size bucket) with tuning on, every candidate
// target is timed on the real launch (the class writes the same values each
// time) and the fastest is recorded.
// the class's lanes-per-quartet layout: tuned once per (class, size bucket) by
// timing the candidates on the main stream, then laid out for the winner
static void eri_class_layout(Context& ctx, EriPlan* P, ClassPlan& c, double* d_out, double* blocks)
{
    int target = 16;
    if (ctx.tune && c.nq > 0) {
        const int bucket = tune_bucket(c.nq);
        if (!tune_get(TUNE_ERI, c.tb, c.tk, bucket, &target)) {
            cudaEvent_t a, b;
            HF_CUDA(cudaEventCreate(&a));
            HF_CUDA(cudaEventCreate(&b));
            float best = 1e30f;
            for (int cand : {4, 8, 16, 32, 64}) {
                layout_class(ctx, c, cand);
                HF_CUDA(cudaEventRecord(a, ctx.stream));
                launch_class(ctx, P, c, MODE_PACKED, d_out, nullptr, blocks);
                HF_CUDA(cudaEventRecord(b, ctx.stream));
                const float ms = elapsed(a, b);
                if (ms < best) {
                    best = ms;
                    target = cand;
                }
            }
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            tune_set(TUNE_ERI, c.tb, c.tk, bucket, target);
        }
    }
    if (c.lane_target != target) layout_class(ctx, c, target);
}

// The ERI pass in two halves: eri_compute_start tunes and lays out the classes
// on the main stream, then launches them over the side streams and returns;
// work the caller queues on the main stream meanwhile runs beside them;
// eri_compute_finish joins the side streams and reports the time.
void eri_compute_start(Context& ctx, EriPlan* P, double* d_out, bool keep_blocks)
{
    P->stats.n_block_elems = 0;
    for (auto& c : P->classes) P->stats.n_block_elems += c.nq * block_size(c.tb, c.tk);
    if (keep_blocks) {
        int64_t total = 0, nqt = 0;
        for (auto& c : P->classes) {
            c.boff = total;
            total += c.nq * block_size(c.tb, c.tk);
            c.qbase = nqt;
            nqt += c.nq;
        }
        P->blocks.alloc(std::max<int64_t>(total, 1), ctx.stream);
        P->qlist.alloc(std::max<int64_t>(nqt, 1), ctx.stream);
    }
    if (!P->ev0) HF_CUDA(cudaEventCreate(&P->ev0));
    if (!P->ev1) HF_CUDA(cudaEventCreate(&P->ev1));
    HF_CUDA(cudaEventRecord(P->ev0, ctx.stream));
    for (int i = (int)P->classes.size() - 1; i >= 0; --i)
        eri_class_layout(ctx, P, P->classes[i], d_out, keep_blocks ? P->blocks.p + P->classes[i].boff : nullptr);
    // the classes write disjoint outputs: spread them over the side streams,
    // heaviest first, so that the small ones fill the SMs around the large ones
    ctx.fork();
    int slot = 0;
    for (int i = (int)P->classes.size() - 1; i >= 0; --i) {
        ClassPlan& c = P->classes[i];
        if (c.nwarps == 0) continue;
        launch_class(ctx, P, c, MODE_PACKED, d_out, nullptr, keep_blocks ? P->blocks.p + c.boff : nullptr,
                     ctx.aux[slot++ % Context::NAUX]);
    }
    // the pass ends with the last class kernel of each side stream (not with
    // whatever the caller queues on the main stream before the join)
    static_assert(Context::NAUX <= 8, "one end event per side stream");
    P->n_ev_end = std::min(slot, (int)Context::NAUX);
    for (int i = 0; i < P->n_ev_end; ++i) {
        if (!P->ev_end[i]) HF_CUDA(cudaEventCreate(&P->ev_end[i]));
        HF_CUDA(cudaEventRecord(P->ev_end[i], ctx.aux[i]));
    }
}

void eri_compute_finish(Context& ctx, EriPlan* P, EriStats* st)
{
    ctx.join();
    HF_CUDA(cudaEventRecord(P->ev1, ctx.stream));
    HF_CUDA(cudaEventSynchronize(P->ev1));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, P->ev0, P->ev1));
    if (P->n_ev_end > 0) {
        ms = 0;
        for (int i = 0; i < P->n_ev_end; ++i) {
            float m = 0;
            HF_CUDA(cudaEventElapsedTime(&m, P->ev0, P->ev_end[i]));
            ms = std::max(ms, m);
        }
    }
    if (st) {
        *st = P->stats;
        st->ms = ms;
    }
}

void eri_compute(Context& ctx, EriPlan* P, double* d_out, bool keep_blocks, EriStats* st)
{
    eri_compute_start(ctx, P, d_out, keep_blocks);
    eri_compute_finish(ctx, P, st);
}



// ------------------------------------------------------------------ batches of molecules
// Several molecules' plans as one: shells, pairs, primitive-pair records, groups
// and prefix sums concatenated with their indices offset, and every class's
// segments from all molecules in one list (each segment tagged with its
// molecule), so that one launch per class computes or digests the quartets of
// every molecule.  Function indices stay local to each molecule.
EriPlan* eri_plan_merge(Context& ctx, const std::vector<EriPlan*>& plans)
{
    cudaStream_t st = ctx.stream;
    auto M = new EriPlan();
    try {
        M->nmol = (int)plans.size();
        std::vector<int> L, np, p0, c0, f0, cfn;
        std::vector<double> xyz, alpha, coef;
        std::vector<int64_t> pref_base(plans.size()), gp_base(plans.size()), pd_base(plans.size());
        int64_t off = 0;
        int pair0 = 0, shell0 = 0;
        for (size_t m = 0; m < plans.size(); ++m) {
            const EriPlan& P = *plans[m];
            const Basis& b = P.basis;
            const int a0 = (int)alpha.size(), cc0 = (int)coef.size(), ff0 = (int)cfn.size();
            M->mol_nbf.push_back(b.nbf);
            M->mol_ns.push_back((int)b.shells.size());
            M->mol_sh0.push_back(shell0);
            for (const Shell& s : b.shells) {
                L.push_back(s.L);
                np.push_back(s.nprim);
                p0.push_back(s.prim0 + a0);
                c0.push_back(s.coef0 + cc0);
                f0.push_back(s.cfn0 + ff0);
                xyz.push_back(s.x);
                xyz.push_back(s.y);
                xyz.push_back(s.z);
            }
            alpha.insert(alpha.end(), b.alpha.begin(), b.alpha.end());
            coef.insert(coef.end(), b.coef.begin(), b.coef.end());
            cfn.insert(cfn.end(), b.comp_fn.begin(), b.comp_fn.end());
            for (int id = 0; id < P.npair; ++id) {
                M->pA.push_back(P.pA[id] + shell0);
                M->pB.push_back(P.pB[id] + shell0);
                M->pK.push_back(P.pK[id]);
                M->pT.push_back(P.pT[id]);
                M->poff.push_back(P.poff[id] + off);
                M->Q.push_back(P.Q[id]);
            }
            gp_base[m] = (int64_t)M->h_gpairs.size();
            for (int g : P.h_gpairs) M->h_gpairs.push_back(g + pair0);
            pref_base[m] = (int64_t)M->h_prefix.size();
            M->h_prefix.insert(M->h_prefix.end(), P.h_prefix.begin(), P.h_prefix.end());
            pd_base[m] = off;
            off += (int64_t)P.pdata.n;
            pair0 += P.npair;
            shell0 += (int)b.shells.size();
            M->stats.n_quartets += P.stats.n_quartets;
            M->stats.n_bf_quartets += P.stats.n_bf_quartets;
            M->stats.n_prim_quartets += P.stats.n_prim_quartets;
            M->stats.flops += P.stats.flops;
        }
        HF_CHECK(M->h_gpairs.size() < (1u << 31) && pair0 < (1 << 30), HFGPU_ERR_UNSUPPORTED,
                 "batch too large for 32-bit pair indexing");
        M->npair = pair0;
        M->sL = to_device(L, st); M->snp = to_device(np, st); M->sp0 = to_device(p0, st);
        M->sc0 = to_device(c0, st); M->scf = to_device(f0, st); M->cfn = to_device(cfn, st);
        M->sxyz = to_device(xyz, st); M->alpha = to_device(alpha, st); M->coef = to_device(coef, st);
        M->dA = to_device(M->pA, st); M->dB = to_device(M->pB, st); M->dK = to_device(M->pK, st);
        M->doff = to_device(M->poff, st);
        M->dQ = to_device(M->Q, st);
        {
            std::vector<int> pm;
            pm.reserve(pair0);
            for (size_t m = 0; m < plans.size(); ++m) pm.insert(pm.end(), plans[m]->npair, (int)m);
            M->pair_mol = to_device(pm, st);
        }
        M->gpairs = to_device(M->h_gpairs, st);
        M->prefix = to_device(M->h_prefix, st);
        M->pdata.alloc(std::max<int64_t>(off, 1), st);
        for (size_t m = 0; m < plans.size(); ++m)
            if (plans[m]->pdata.n)
                HF_CUDA(cudaMemcpyAsync(M->pdata.p + pd_base[m], plans[m]->pdata.p, plans[m]->pdata.n * sizeof(double),
                                        cudaMemcpyDeviceToDevice, st));
        for (int tb = 0; tb < NPTYPE; tb++)
            for (int tk = tb; tk < NPTYPE; tk++) {
                ClassPlan c;
                c.tb = tb;
                c.tk = tk;
                for (size_t m = 0; m < plans.size(); ++m)
                    for (const ClassPlan& pc : plans[m]->classes) {
                        if (pc.tb != tb || pc.tk != tk) continue;
                        for (size_t i = 0; i < pc.segs.size(); ++i) {
                            Seg s = pc.segs[i];
                            s.pref0 += pref_base[m];
                            s.bra0 += (int)gp_base[m];
                            s.ket0 += (int)gp_base[m];
                            s.mol = (int)m;
                            s.qoff = c.nq;
                            c.nq += s.nq;
                            c.segs.push_back(s);
                            c.kprod.push_back(pc.kprod[i]);
                        }
                    }
                if (c.segs.empty()) continue;
                HF_CHECK(c.nq < (1ll << 31), HFGPU_ERR_UNSUPPORTED, "quartet class too large for 32-bit indexing");
                c.dsegs = to_device(c.segs, st);
                layout_class(ctx, c, 16);
                M->classes.push_back(std::move(c));
            }
        HF_CUDA(cudaStreamSynchronize(st));
        return M;
    } catch (...) {
        delete M;
        throw;
    }
}

// largest |P| of every shell pair of every molecule with a screened build
__global__ void batch_dmax_kernel(int nmol, const int64_t* __restrict__ dm_prefix, const int* __restrict__ L,
                                  const int* __restrict__ cfn0, const int* __restrict__ comp_fn,
                                  const int* __restrict__ mol_n, const int* __restrict__ mol_ns,
                                  const int* __restrict__ mol_sh0, const double* const* __restrict__ mol_P,
                                  const double* __restrict__ mol_screen, double* __restrict__ Dm)
{
    const int64_t total = dm_prefix[nmol];
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = nmol - 1;  // last molecule with dm_prefix <= idx
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (dm_prefix[mid] <= idx) lo = mid; else hi = mid - 1;
        }
        if (mol_screen[lo] <= 0.0) continue;
        const int ns = mol_ns[lo], n = mol_n[lo];
        const int64_t e = idx - dm_prefix[lo];
        const int s1 = mol_sh0[lo] + (int)(e / ns), s2 = mol_sh0[lo] + (int)(e % ns);
        const double* P = mol_P[lo];
        double m = 0.0;
        for (int i = 0; i < ncart(L[s1]); ++i) {
            const int f = comp_fn[cfn0[s1] + i];
            if (f < 0) continue;
            for (int j = 0; j < ncart(L[s2]); ++j) {
                const int g = comp_fn[cfn0[s2] + j];
                if (g >= 0) m = fmax(m, fabs(P[f + (int64_t)g * n]));
            }
        }
        Dm[idx] = m;
    }
}

// G_m = Gh_m + Gh_m^T for every molecule of the build
__global__ void batch_sym_kernel(int nmol, const int64_t* __restrict__ nn_prefix, const int* __restrict__ mol_n,
                                 const double* __restrict__ Gh, double* const* __restrict__ mol_G,
                                 const double* __restrict__ mol_screen)
{
    const int64_t total = nn_prefix[nmol];
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = nmol - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (nn_prefix[mid] <= idx) lo = mid; else hi = mid - 1;
        }
        if (mol_screen[lo] < 0.0) continue;
        const int n = mol_n[lo];
        const int64_t e = idx - nn_prefix[lo];
        const int i = (int)(e % n), j = (int)(e / n);
        const double* gh = Gh + nn_prefix[lo];
        mol_G[lo][e] = gh[e] + gh[j + (int64_t)i * n];
    }
}

void BatchDigest::setup(Context& ctx, const EriPlan* P, cudaStream_t s)
{
    nmol = P->nmol;
    std::vector<int64_t> nnp(nmol + 1, 0), dmp(nmol + 1, 0);
    for (int m = 0; m < nmol; ++m) {
        nnp[m + 1] = nnp[m] + (int64_t)P->mol_nbf[m] * P->mol_nbf[m];
        dmp[m + 1] = dmp[m] + (int64_t)P->mol_ns[m] * P->mol_ns[m];
    }
    nn_prefix = to_device(nnp, s);
    dm_prefix = to_device(dmp, s);
    mol_n = to_device(P->mol_nbf, s);
    mol_ns = to_device(P->mol_ns, s);
    mol_sh0 = to_device(P->mol_sh0, s);
    Gh.alloc(std::max<int64_t>(nnp[nmol], 1), s);
    Dm.alloc(std::max<int64_t>(dmp[nmol], 1), s);
    std::vector<double*> gh(nmol);
    std::vector<const double*> dm(nmol);
    for (int m = 0; m < nmol; ++m) {
        gh[m] = Gh.p + nnp[m];
        dm[m] = Dm.p + dmp[m];
    }
    mol_Gh = to_device(gh, s);
    mol_Dm = to_device(dm, s);
    mol_P.alloc(nmol, s);
    mol_G.alloc(nmol, s);
    mol_screen.alloc(nmol, s);
    HF_CUDA(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming));
    HF_CUDA(cudaMallocHost((void**)&h_P, nmol * sizeof(const double*)));
    HF_CUDA(cudaMallocHost((void**)&h_G, nmol * sizeof(double*)));
    HF_CUDA(cudaMallocHost((void**)&h_screen, nmol * sizeof(double)));
    for (int m = 0; m < nmol; ++m) {
        h_P[m] = nullptr;
        h_G[m] = nullptr;
        h_screen[m] = -1.0;
    }
}

void BatchDigest::wait_tables()
{
    if (copied) HF_CUDA(cudaEventSynchronize(copied));
}

BatchDigest::~BatchDigest()
{
    if (copied) cudaEventDestroy(copied);
    if (exec) cudaGraphExecDestroy(exec);
    if (h_P) cudaFreeHost((void*)h_P);
    if (h_G) cudaFreeHost(h_G);
    if (h_screen) cudaFreeHost(h_screen);
}

// One Fock build for every molecule whose h_screen >= 0: Gh zeroed, shell-pair
// maxima for the screened ones, one digest launch per quartet class over all
// molecules' quartets, and the symmetrisation into each molecule's G.
static void batch_digest_launches(Context& ctx, EriPlan* P, BatchDigest& t, cudaStream_t s)
{
    HF_CUDA(cudaMemsetAsync(t.Gh.p, 0, t.Gh.n * sizeof(double), s));
    const int64_t dm_total = t.Dm.n, nn_total = t.Gh.n;
    const unsigned gd = (unsigned)std::max<int64_t>(1, std::min<int64_t>((dm_total + 255) / 256, ctx.num_sms * 8));
    batch_dmax_kernel<<<gd, 256, 0, s>>>(t.nmol, t.dm_prefix.p, P->sL.p, P->scf.p, P->cfn.p, t.mol_n.p, t.mol_ns.p,
                                        t.mol_sh0.p, t.mol_P.p, t.mol_screen.p, t.Dm.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
    // the classes are independent until the symmetrisation: spread over the side
    // streams (inside a capture these become parallel branches of the graph)
    HF_CUDA(cudaEventRecord(ctx.fork_ev, s));
    for (int i = 0; i < Context::NAUX; ++i) HF_CUDA(cudaStreamWaitEvent(ctx.aux[i], ctx.fork_ev, 0));
    int slot = 0;
    for (int ci = (int)P->classes.size() - 1; ci >= 0; --ci) {
        auto& c = P->classes[ci];
        if (c.nq == 0) continue;
        DigestArgs a;
        a.sh = P->shdev();
        a.pr = P->prdev();
        a.gpairs = P->gpairs.p;
        a.prefix = P->prefix.p;
        a.list = nullptr;
        a.segs = c.dsegs.p;
        a.nseg = (int)c.segs.size();
        a.nq = c.nq;
        a.blocks = P->blocks.p + c.boff;
        a.P = nullptr;
        a.n = 0;
        a.Gh = nullptr;
        a.screen = 0.0;
        a.Q = P->dQ.p;
        a.Dm = nullptr;
        a.ns = 0;
        a.mol_n = t.mol_n.p;
        a.mol_P = t.mol_P.p;
        a.mol_Gh = t.mol_Gh.p;
        a.mol_screen = t.mol_screen.p;
        a.mol_Dm = t.mol_Dm.p;
        a.mol_ns = t.mol_ns.p;
        a.mol_sh0 = t.mol_sh0.p;
        a.qlist = P->qlist.p ? P->qlist.p + c.qbase : nullptr;
        a.pair_mol = P->pair_mol.p;
        int split = digest_split(c);
        if (ctx.tune) tune_get(TUNE_DIGEST, c.tb, c.tk, tune_bucket(c.nq), &split);
        a.split = split;
        // captured once for all builds, screened or not
        a.rounds = digest_rounds(ctx, c, split, true);
        launch_digest(c, a, ctx.aux[slot++ % Context::NAUX]);
    }
    for (int i = 0; i < Context::NAUX; ++i) {
        HF_CUDA(cudaEventRecord(ctx.join_ev[i], ctx.aux[i]));
        HF_CUDA(cudaStreamWaitEvent(s, ctx.join_ev[i], 0));
    }
    const unsigned gs = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nn_total + 255) / 256, ctx.num_sms * 8));
    batch_sym_kernel<<<gs, 256, 0, s>>>(t.nmol, t.nn_prefix.p, t.mol_n.p, t.Gh.p, t.mol_G.p, t.mol_screen.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

void eri_digest_batch(Context& ctx, EriPlan* P, BatchDigest& t, cudaStream_t s)
{
    HF_CHECK(P->blocks.p != nullptr && P->nmol == t.nmol, HFGPU_ERR_INVALID, "eri_digest_batch: plan and tables differ");
    // this build's densities, outputs and screens
    HF_CUDA(cudaMemcpyAsync(t.mol_P.p, t.h_P, t.nmol * sizeof(const double*), cudaMemcpyHostToDevice, s));
    HF_CUDA(cudaMemcpyAsync(t.mol_G.p, t.h_G, t.nmol * sizeof(double*), cudaMemcpyHostToDevice, s));
    HF_CUDA(cudaMemcpyAsync(t.mol_screen.p, t.h_screen, t.nmol * sizeof(double), cudaMemcpyHostToDevice, s));
    HF_CUDA(cudaEventRecord(t.copied, s));
    if (!t.exec) {
        // the launches of a build are the same every iteration: captured once into a
        // CUDA graph and replayed (the tables above are read from device memory)
        const int64_t before = launches_counted();
        cudaGraph_t g = nullptr;
        HF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
            batch_digest_launches(ctx, P, t, s);
        } catch (...) {
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        HF_CUDA(cudaStreamEndCapture(s, &g));
        t.graph_kernels = launches_counted() - before;
        count_launch(-(int)t.graph_kernels);  // captured, not yet run
        const cudaError_t e = cudaGraphInstantiate(&t.exec, g, 0);
        cudaGraphDestroy(g);
        HF_CUDA(e);
    }
    HF_CUDA(cudaGraphLaunch(t.exec, s));
    count_launch((int)t.graph_kernels);
}

}  // namespace hfgpu
