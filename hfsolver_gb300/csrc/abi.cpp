// extern "C" entry points of libhfgpu (declared in include/hfgpu.h).
#include <chrono>
#include <cstdlib>
#include <memory>
#include <cmath>
#include <cstring>
#include <new>
#include <atomic>
#include <thread>
#include <algorithm>
#include <string>
#include <vector>

#include "autotune.h"
#include "batch.h"
#include "eigh.h"
#include "internal.h"
#include "scf.h"
#include "tcgemm.h"

using namespace hfgpu;

namespace {

template <class F>
int guard(F&& f)
{
    try {
        f();
        return HFGPU_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return HFGPU_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return HFGPU_ERR_CUDA;
    }
}

struct Timer {
    cudaEvent_t a, b;
    cudaStream_t s;
    explicit Timer(cudaStream_t st) : s(st)
    {
        HF_CUDA(cudaEventCreate(&a));
        HF_CUDA(cudaEventCreate(&b));
        HF_CUDA(cudaEventRecord(a, s));
    }
    double ms()
    {
        HF_CUDA(cudaEventRecord(b, s));
        HF_CUDA(cudaEventSynchronize(b));
        float t = 0;
        HF_CUDA(cudaEventElapsedTime(&t, a, b));
        return t;
    }
    ~Timer()
    {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

void check_ptr(const void* p, const char* name)
{
    HF_CHECK(p != nullptr, HFGPU_ERR_INVALID, std::string(name) + " is NULL");
}

void onee_dropin(int which, int nbf, const int* nprim, const int* istart, const double* xc, const double* yc,
                 const double* zc, const int* lp, const int* mp, const int* np, int n2, const double* coef,
                 const double* alpha, int nat, const int* atno, const double* x, const double* y, const double* z,
                 double* out)
{
    check_ptr(out, "output");
    Basis b = basis_from_functions(nbf, nprim, istart, xc, yc, zc, lp, mp, np, n2, coef, alpha);
    Context& ctx = context();
    std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
    DBuf<double> d((size_t)nbf * nbf, ctx.stream);
    onee_compute(ctx, b, nat, atno, x, y, z, which == 0 ? d.p : nullptr, which == 1 ? d.p : nullptr,
                 which == 2 ? d.p : nullptr);
    d.download(out, (size_t)nbf * nbf);
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
}

void ints_dropin(const Basis& b, double* Ints, double schwarz, EriStats* st)
{
    Context& ctx = context();
    std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
    const int64_t np = packed_size(b.nbf);
    DBuf<double> d(np, ctx.stream);
    d.zero();
    EriPlan* plan = eri_plan_create(ctx, b, schwarz);
    try {
        eri_compute_packed(ctx, plan, d.p, st);
    } catch (...) {
        eri_plan_destroy(plan);
        throw;
    }
    eri_plan_destroy(plan);
    d.download(Ints, np);
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
}

}  // namespace

// a molecule's place in a wave of hfgpu_rhf_batch's fused mode (batch.h)
struct BatchMember {
    BatchWave* wave;
    int mol;
};

static void rhf_impl(int natoms, const int* atno, const double* xyz, const hfgpu_options* opt_in, hfgpu_result* res,
                     double* C, double* lam, int& conv, int& nscf, double* grad = nullptr,
                     Context* ctx_in = nullptr, BatchMember* bm = nullptr)
{
        // a wave's member leaves it however this call ends (its builds go on without it)
        struct WaveExit {
            BatchMember* b;
            void now() { if (b) b->wave->leave(b->mol); b = nullptr; }
            ~WaveExit() { now(); }
        } wave_exit{bm};
        check_ptr(atno, "atno"); check_ptr(xyz, "xyz"); check_ptr(res, "res");
        hfgpu_options opt;
        if (opt_in) opt = *opt_in; else hfgpu_default_options(&opt);
        nscf = opt.nscf;
        HF_CHECK(opt.nscf >= 1, HFGPU_ERR_INVALID, "nscf must be >= 1");
        HF_CHECK(opt.mp2 >= HFGPU_MP2_NONE && opt.mp2 <= HFGPU_MP2_SPLIT_BF16, HFGPU_ERR_INVALID,
                 "unknown MP2 precision");
        std::memset(res, 0, sizeof(*res));
        Basis b = build_basis(natoms, atno, xyz);  // validates the input before any device work
        Context& ctx = ctx_in ? *ctx_in : context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        cudaStream_t st = ctx.stream;
        ctx.settle_timers();  // drop timers a failed earlier call may have left
        ctx.trace_begin();
        ctx.stat_fock_ms = ctx.stat_tc_ms = ctx.stat_tc_flops = 0;
        ctx.stat_tc_step1_ms = ctx.stat_tc_step1_n = 0;
        ctx.stat_fock_full_ms = ctx.stat_fock_full_n = 0;
        ctx.tune = opt.autotune != 0 || tune_env_enabled();
        Timer total(st);
        const int n = b.nbf;
        int nelec = 0;
        for (int i = 0; i < natoms; i++) nelec += atno[i];
        const int nocc = nelec / 2;
        const size_t nn = (size_t)n * n;
        res->nbf = n;
        res->nocc = nocc;
        res->nshell = (int)b.shells.size();
        std::vector<double> x(natoms), y(natoms), z(natoms);
        for (int i = 0; i < natoms; i++) { x[i] = xyz[3 * i]; y[i] = xyz[3 * i + 1]; z[i] = xyz[3 * i + 2]; }
        DBuf<double> dS(nn, st), dT(nn, st), dV(nn, st), dH(nn, st);
        // the one-electron integrals run on a side stream, under the ERI plan's
        // host work (pair lists, quartet classes); joined before H is formed
        ctx.fork();
        onee_compute(ctx, b, natoms, atno, x.data(), y.data(), z.data(), dS.p, dT.p, dV.p, ctx.aux[0]);
        // integrals, resident in HBM for the whole SCF (in a wave: the wave's arrays)
        DBuf<double> dI;
        if (!bm) {
            dI.alloc(packed_size(n), st);
            dI.zero();
        }
        const double* d_int2 = dI.p;
        EriStats es;
        std::unique_ptr<EriPlan, void (*)(EriPlan*)> plan(eri_plan_create(ctx, b, opt.schwarz), eri_plan_destroy);
        ctx.join();
        {
            const double one = 1.0;
            HF_CUBLAS(cublasDgeam(ctx.blas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, &one, dT.p, n, &one, dV.p, n, dH.p, n));
        }
        res->ms_setup = total.ms();
        ctx.trace_mark("one-electron + plan");
        // the packed array feeds MBPT2; the screened quartet blocks feed every Fock build.
        // One molecule: the ERI classes run on the side streams while the SCF queues
        // its set-up on the main stream (ScfIn::begin / end below).
        struct EriHook {
            Context* ctx;
            EriPlan* plan;
            double* out;
            EriStats* es;
        } hook{&ctx, plan.get(), dI.p, &es};
        if (bm) {
            d_int2 = bm->wave->eri_rendezvous(bm->mol, ctx, plan.get(), &es.ms);
            const double ms = es.ms;
            es = eri_plan_stats(plan.get());
            es.ms = ms;
            ctx.trace_mark("eri");
        }
        // SCF
        Timer ts(st);
        DBuf<double> dC(nn, st), dP(nn, st), dL(n, st);
        ScfIn in;
        in.n = n; in.nocc = nocc; in.nscf = opt.nscf; in.dH = dH.p; in.dS = dS.p; in.d_int2 = d_int2;
        in.tolE = opt.tolE; in.tolP = opt.tolP; in.alpha = opt.mix_alpha;
        in.accel = opt.scf_accel; in.diis_size = opt.diis_size > 0 ? opt.diis_size : 8;
        in.purify = opt.purify != 0;
        in.eigensolver = opt.eigensolver;
        in.direct_jk = [](Context& c, void* user, const double* P, double* G, double screen) {
            eri_digest(c, (EriPlan*)user, P, G, screen);
        };
        // density-difference builds skip quartets whose bounded contribution is below
        // 1e-10 (or the Schwarz threshold, if larger); the full builds of the last
        // iterations remove what they left out before convergence is accepted
        if (opt.incremental) in.inc_screen = std::max(opt.schwarz, 1e-10);
        in.direct_ctx = plan.get();
        if (!bm) {
            in.begin = [](void* u) {
                auto* h = (EriHook*)u;
                eri_compute_start(*h->ctx, h->plan, h->out, true);
            };
            in.end = [](void* u) {
                auto* h = (EriHook*)u;
                eri_compute_finish(*h->ctx, h->plan, h->es);
                h->ctx->trace_mark("eri");
            };
            in.hook_user = &hook;
        }
        if (bm) {  // Fock builds shared with the rest of the wave
            in.direct_jk = [](Context& c, void* user, const double* P, double* G, double screen) {
                auto* m = (BatchMember*)user;
                m->wave->digest(m->mol, c, P, G, screen);
            };
            in.direct_ctx = bm;
        }
        DBuf<double> dP0;
        if (opt.guess == 1) {  // superposition of atomic densities instead of P = 0
            dP0.alloc(nn, st);
            sad_guess(ctx, natoms, atno, n, dP0.p);
            in.dP0 = dP0.p;
            ctx.trace_mark("guess");
        }
        ScfOut so = run_scf(ctx, in, dC.p, dP.p, dL.p);
        res->ms_eri = es.ms;
        res->n_quartets = es.n_quartets;
        res->n_bf_quartets = es.n_bf_quartets;
        res->n_prim_quartets = es.n_prim_quartets;
        res->eri_flops = es.flops;
        if (bm) res->ms_fock = bm->wave->fock_ms();
        wave_exit.now();
        res->ms_scf = ts.ms() - (bm ? 0.0 : es.ms);  // the ERI pass ran inside, beside the SCF's set-up
        conv = so.converged;
        double Enuc = 0;
        for (int i = 0; i < natoms; i++)
            for (int j = 0; j < i; j++) {
                double dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1],
                       dz = xyz[3 * i + 2] - xyz[3 * j + 2];
                Enuc += atno[i] * atno[j] / std::sqrt(dx * dx + dy * dy + dz * dz);
            }
        res->E0 = so.E0;
        res->Enuc = Enuc;
        res->Etot = so.E0 + Enuc;
        res->Ekin = device_dot(ctx, (int64_t)nn, dP.p, dT.p);
        res->dP = so.dP;
        res->niter = so.niter;
        // MBPT2
        if (conv && opt.mp2 != HFGPU_MP2_NONE) {
            Timer tm(st);
            const int mo = opt.mp2_nocc > 0 ? opt.mp2_nocc : nocc;
            HF_CHECK(mo <= n, HFGPU_ERR_INVALID, "mp2_nocc larger than the basis");
            const int mv = n - mo;
            if (mo > 0 && mv > 0 && opt.mp2 == HFGPU_MP2_SPLIT_BF16) {
                res->E2 = mp2_energy_mixed(ctx, n, d_int2, dC.p, mo, dL.p);
            } else if (mo > 0 && mv > 0) {
                DBuf<double> iajb((size_t)mo * mv * mo * mv, st);
                ao2mo_fp64(ctx, n, d_int2, dC.p, mo, dC.p + (size_t)n * mo, mv, iajb.p);
                res->E2 = mp2_energy(ctx, mo, mv, iajb.p, dL.p);
            }
            res->ms_mp2 = tm.ms();
            ctx.trace_mark("mp2");
        }
        // analytic nuclear gradient at the converged orbitals
        if (conv && grad) {
            rhf_gradient(ctx, plan.get(), natoms, atno, xyz, dC.p, dL.p, nocc, grad, &res->ms_grad, &res->ms_grad_eri);
            ctx.trace_mark("gradient");
        }
        if (C) dC.download(C, nn);
        if (lam) dL.download(lam, n);
        HF_CUDA(cudaStreamSynchronize(st));
        res->ms_total = total.ms();
        ctx.trace_mark("download");
        ctx.trace_report();
        ctx.settle_timers();
        if (!bm) res->ms_fock = ctx.stat_fock_ms;
        res->ms_fock_full = ctx.stat_fock_full_ms;
        res->n_fock_full = ctx.stat_fock_full_n;
        res->block_elems = (double)es.n_block_elems;
        res->ms_tcgemm = ctx.stat_tc_ms;
        res->tc_flops = ctx.stat_tc_flops;
        res->ms_tc_step1 = ctx.stat_tc_step1_ms;
        res->n_tc_step1 = ctx.stat_tc_step1_n;
}

static void streams_batch(int nmol, const int* natoms, const int* atno, const double* xyz,
                          const std::vector<int64_t>& a0, const hfgpu_options* opt, hfgpu_result* res,
                          std::vector<int>& rc, std::vector<std::string>& err, int dev);
static void fused_batch(int nmol, const int* natoms, const int* atno, const double* xyz,
                        const std::vector<int64_t>& a0, const hfgpu_options* opt, hfgpu_result* res,
                        std::vector<int>& rc, std::vector<std::string>& err, int dev);

extern "C" {

int hfgpu_getS(int nbf, const int* nprim, const int* istart, const double* xc, const double* yc, const double* zc,
               const int* lp, const int* mp, const int* np, int n2, const double* coef, const double* alpha,
               double* S)
{
    return guard([&] {
        onee_dropin(0, nbf, nprim, istart, xc, yc, zc, lp, mp, np, n2, coef, alpha, 0, nullptr, nullptr, nullptr,
                    nullptr, S);
    });
}

int hfgpu_getT(int nbf, const int* nprim, const int* istart, const double* xc, const double* yc, const double* zc,
               const int* lp, const int* mp, const int* np, int n2, const double* coef, const double* alpha,
               double* T)
{
    return guard([&] {
        onee_dropin(1, nbf, nprim, istart, xc, yc, zc, lp, mp, np, n2, coef, alpha, 0, nullptr, nullptr, nullptr,
                    nullptr, T);
    });
}

int hfgpu_getV(int nbf, const int* nprim, const int* istart, const double* xc, const double* yc, const double* zc,
               const int* lp, const int* mp, const int* np, int n2, const double* coef, const double* alpha, int nat,
               const int* atno, const double* x, const double* y, const double* z, double* V)
{
    return guard([&] {
        HF_CHECK(nat >= 0, HFGPU_ERR_INVALID, "nat must be >= 0");
        for (int i = 0; i < nat; i++)
            HF_CHECK(std::isfinite(x[i]) && std::isfinite(y[i]) && std::isfinite(z[i]), HFGPU_ERR_INVALID,
                     "non-finite nuclear coordinate");
        onee_dropin(2, nbf, nprim, istart, xc, yc, zc, lp, mp, np, n2, coef, alpha, nat, atno, x, y, z, V);
    });
}

int hfgpu_getInts(int nbf, const int* nprim, const int* istart, const double* xc, const double* yc,
                  const double* zc, const int* lp, const int* mp, const int* np, int n2, const double* coef,
                  const double* alpha, double* Ints)
{
    return guard([&] {
        check_ptr(Ints, "Ints");
        Basis b = basis_from_functions(nbf, nprim, istart, xc, yc, zc, lp, mp, np, n2, coef, alpha);
        ints_dropin(b, Ints, 0.0, nullptr);
    });
}

int hfgpu_getints2(int n, const int* nprim, const int* istart, const double* center, const int* power, int n2,
                   const double* coef, const double* alpha, double* int2, int64_t nint2)
{
    return guard([&] {
        HF_CHECK(n >= 1, HFGPU_ERR_INVALID, "n must be >= 1");
        HF_CHECK(nint2 == packed_size(n), HFGPU_ERR_INVALID,
                 "size(int2) must be m(m+1)/2 with m = n(n+1)/2");
        check_ptr(int2, "int2");
        std::vector<int> st0(n), lp(n), mp(n), npw(n);
        std::vector<double> xc(n), yc(n), zc(n);
        for (int i = 0; i < n; i++) {
            st0[i] = istart[i] - 1;
            xc[i] = center[3 * i]; yc[i] = center[3 * i + 1]; zc[i] = center[3 * i + 2];
            lp[i] = power[3 * i]; mp[i] = power[3 * i + 1]; npw[i] = power[3 * i + 2];
        }
        Basis b = basis_from_functions(n, nprim, st0.data(), xc.data(), yc.data(), zc.data(), lp.data(), mp.data(),
                                       npw.data(), n2, coef, alpha);
        ints_dropin(b, int2, 0.0, nullptr);
    });
}

int hfgpu_doscf(int n, const double* H, const double* int2, const double* S, int nocc, int nscf, double tolE,
                double tolP, double alpha, double* C, double* P, double* lam, double* E0, int* niter)
{
    int conv = 1;
    int rc = guard([&] {
        HF_CHECK(n >= 1 && nocc >= 0 && nocc <= n && nscf >= 1, HFGPU_ERR_INVALID, "invalid sizes");
        check_ptr(H, "H"); check_ptr(int2, "int2"); check_ptr(S, "S");
        check_ptr(C, "C"); check_ptr(P, "P"); check_ptr(lam, "lam"); check_ptr(E0, "E0");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const size_t nn = (size_t)n * n;
        DBuf<double> dH(nn, ctx.stream), dS(nn, ctx.stream), dI(packed_size(n), ctx.stream);
        DBuf<double> dC(nn, ctx.stream), dP(nn, ctx.stream), dL(n, ctx.stream);
        dH.upload(H, nn); dS.upload(S, nn); dI.upload(int2, packed_size(n));
        ScfIn in;
        in.n = n; in.nocc = nocc; in.nscf = nscf; in.dH = dH.p; in.dS = dS.p; in.d_int2 = dI.p;
        in.tolE = tolE; in.tolP = tolP; in.alpha = alpha;
        ScfOut o = run_scf(ctx, in, dC.p, dP.p, dL.p);
        dC.download(C, nn); dP.download(P, nn); dL.download(lam, n);
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
        *E0 = o.E0;
        if (niter) *niter = o.niter;
        conv = o.converged;
    });
    if (rc == HFGPU_OK && !conv) {
        set_last_error("SCF did not converge in " + std::to_string(nscf) + " iterations.");
        return HFGPU_ERR_NOT_CONVERGED;
    }
    return rc;
}

int hfgpu_eigh(int n, const double* A, const double* B, double* lam, double* C)
{
    return guard([&] {
        HF_CHECK(n >= 1, HFGPU_ERR_INVALID, "n must be >= 1");
        check_ptr(A, "A"); check_ptr(B, "B"); check_ptr(lam, "lam"); check_ptr(C, "C");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const size_t nn = (size_t)n * n;
        DBuf<double> dA(nn, ctx.stream), dB(nn, ctx.stream), dC(nn, ctx.stream), dL(n, ctx.stream);
        dA.upload(A, nn);
        dB.upload(B, nn);
        eigh_generalized(ctx, n, dA.p, dB.p, dC.p, dL.p, 0);
        dC.download(C, nn);
        dL.download(lam, n);
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
    });
}

double hfgpu_md_flops(int la, int lb, int lc, int ld)
{
    if (la < 0 || lb < 0 || lc < 0 || ld < 0) return 0.0;
    return md_flops(la, lb, lc, ld);
}

int hfgpu_tridiag_eigen(int n, const double* d, const double* e, double* lam, double* Z)
{
    return guard([&] {
        HF_CHECK(n >= 1, HFGPU_ERR_INVALID, "n must be >= 1");
        check_ptr(d, "d"); check_ptr(lam, "lam"); check_ptr(Z, "Z");
        if (n > 1) check_ptr(e, "e");
        for (int i = 0; i < n; ++i) HF_CHECK(std::isfinite(d[i]), HFGPU_ERR_INVALID, "non-finite diagonal");
        for (int i = 0; i + 1 < n; ++i) HF_CHECK(std::isfinite(e[i]), HFGPU_ERR_INVALID, "non-finite off-diagonal");
        tridiag_eigen(n, d, e, lam, Z, n);
    });
}

int hfgpu_formG(int n, const double* P, const double* int2, double* G)
{
    return guard([&] {
        HF_CHECK(n >= 1, HFGPU_ERR_INVALID, "n must be >= 1");
        check_ptr(P, "P"); check_ptr(int2, "int2"); check_ptr(G, "G");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const size_t nn = (size_t)n * n;
        DBuf<double> dP(nn, ctx.stream), dI(packed_size(n), ctx.stream), dG(nn, ctx.stream);
        dP.upload(P, nn);
        dI.upload(int2, packed_size(n));
        jk_from_packed(ctx, n, dI.p, dP.p, dG.p);
        dG.download(G, nn);
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
    });
}

int hfgpu_jk(int nbf, const int* nprim, const int* istart, const double* xc, const double* yc, const double* zc,
             const int* lp, const int* mp, const int* np, int n2, const double* coef, const double* alpha,
             const double* P, double schwarz, double* J, double* K)
{
    return guard([&] {
        check_ptr(P, "P"); check_ptr(J, "J"); check_ptr(K, "K");
        HF_CHECK(schwarz >= 0, HFGPU_ERR_INVALID, "schwarz must be >= 0");
        Basis b = basis_from_functions(nbf, nprim, istart, xc, yc, zc, lp, mp, np, n2, coef, alpha);
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const size_t nn = (size_t)nbf * nbf;
        DBuf<double> dI(packed_size(nbf), ctx.stream), dP(nn, ctx.stream), dJ(nn, ctx.stream), dK(nn, ctx.stream);
        dI.zero();
        dP.upload(P, nn);
        EriPlan* plan = eri_plan_create(ctx, b, schwarz);
        try {
            eri_compute_packed(ctx, plan, dI.p, nullptr);
        } catch (...) {
            eri_plan_destroy(plan);
            throw;
        }
        eri_plan_destroy(plan);
        jk_separate_from_packed(ctx, nbf, dI.p, dP.p, dJ.p, dK.p);
        dJ.download(J, nn);
        dK.download(K, nn);
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
    });
}

int hfgpu_mp2_energy(int n, const double* int2, const double* C, const double* lam, int nocc, int precision,
                     double* E2)
{
    return guard([&] {
        HF_CHECK(n >= 1 && nocc >= 0 && nocc <= n, HFGPU_ERR_INVALID, "invalid sizes");
        HF_CHECK(precision == HFGPU_MP2_FP64 || precision == HFGPU_MP2_SPLIT_BF16, HFGPU_ERR_INVALID,
                 "precision must be HFGPU_MP2_FP64 or HFGPU_MP2_SPLIT_BF16");
        check_ptr(int2, "int2"); check_ptr(C, "C"); check_ptr(lam, "lam"); check_ptr(E2, "E2");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const size_t nn = (size_t)n * n;
        DBuf<double> dI(packed_size(n), ctx.stream), dC(nn, ctx.stream), dL(n, ctx.stream);
        dI.upload(int2, packed_size(n));
        dC.upload(C, nn);
        dL.upload(lam, n);
        const int v = n - nocc;
        double e = 0.0;
        if (nocc > 0 && v > 0) {
            if (precision == HFGPU_MP2_SPLIT_BF16) {
                e = mp2_energy_mixed(ctx, n, dI.p, dC.p, nocc, dL.p);
            } else {
                DBuf<double> iajb((size_t)nocc * v * nocc * v, ctx.stream);
                ao2mo_fp64(ctx, n, dI.p, dC.p, nocc, dC.p + (size_t)n * nocc, v, iajb.p);
                e = mp2_energy(ctx, nocc, v, iajb.p, dL.p);
            }
        }
        *E2 = e;
    });
}

int hfgpu_transform_int2(int n, const double* int2, const double* C, double* moint2)
{
    return guard([&] {
        HF_CHECK(n >= 1, HFGPU_ERR_INVALID, "n must be >= 1");
        check_ptr(int2, "int2"); check_ptr(C, "C"); check_ptr(moint2, "moint2");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const int64_t np = packed_size(n);
        DBuf<double> dI(np, ctx.stream), dC((size_t)n * n, ctx.stream), dM(np, ctx.stream);
        dI.upload(int2, np);
        dC.upload(C, (size_t)n * n);
        transform_packed(ctx, n, dI.p, dC.p, dM.p);
        dM.download(moint2, np);
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
    });
}

int hfgpu_mbpt2(int n, const double* moint2, const double* lam, int nocc, double* E2)
{
    return guard([&] {
        HF_CHECK(n >= 1 && nocc >= 0 && nocc <= n, HFGPU_ERR_INVALID, "invalid sizes");
        check_ptr(moint2, "moint2"); check_ptr(lam, "lam"); check_ptr(E2, "E2");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const int64_t np = packed_size(n);
        DBuf<double> dM(np, ctx.stream), dL(n, ctx.stream);
        dM.upload(moint2, np);
        dL.upload(lam, n);
        *E2 = mbpt2_packed(ctx, n, dM.p, dL.p, nocc);
    });
}

int hfgpu_mbpt3(int n, const double* moint2, const double* lam, int nocc, double* E3)
{
    return guard([&] {
        HF_CHECK(n >= 1 && nocc >= 0 && nocc <= n, HFGPU_ERR_INVALID, "invalid sizes");
        check_ptr(moint2, "moint2"); check_ptr(lam, "lam"); check_ptr(E3, "E3");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const int64_t np = packed_size(n);
        DBuf<double> dM(np, ctx.stream), dL(n, ctx.stream);
        dM.upload(moint2, np);
        dL.upload(lam, n);
        *E3 = mbpt3_packed(ctx, n, dM.p, dL.p, nocc);
    });
}

int hfgpu_find_pole_diag(int n, const double* moint2, const double* lam, int nocc, int i, int nscf, double tolE,
                         double* E, int* niter)
{
    return guard([&] {
        HF_CHECK(n >= 2 && nocc >= 1 && nocc < n, HFGPU_ERR_INVALID, "find_pole_diag: need 1 <= nocc < n");
        HF_CHECK(i >= 1 && i <= n, HFGPU_ERR_INVALID, "find_pole_diag: i is a 1-based orbital index in [1, n]");
        HF_CHECK(nscf >= 1 && tolE > 0, HFGPU_ERR_INVALID, "find_pole_diag: need nscf >= 1 and tolE > 0");
        check_ptr(moint2, "moint2"); check_ptr(lam, "lam"); check_ptr(E, "E");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        const int64_t np = packed_size(n);
        DBuf<double> dM(np, ctx.stream), dL(n, ctx.stream);
        dM.upload(moint2, np);
        dL.upload(lam, n);
        int it = 0;
        *E = find_pole_diag(ctx, n, dM.p, dL.p, nocc, i - 1, nscf, tolE, &it);
        if (niter) *niter = it;
    });
}

int hfgpu_dgemm_sliced(int64_t M, int N, int K, const double* A, const double* Bt, double* C)
{
    return guard([&] {
        HF_CHECK(M >= 1 && N >= 1 && K >= 1 && K <= 512, HFGPU_ERR_INVALID, "need M, N >= 1 and 1 <= K <= 512");
        check_ptr(A, "A"); check_ptr(Bt, "Bt"); check_ptr(C, "C");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        DBuf<double> dA((size_t)M * K, ctx.stream), dB((size_t)N * K, ctx.stream), dC((size_t)M * N, ctx.stream);
        dA.upload(A, (size_t)M * K);
        dB.upload(Bt, (size_t)N * K);
        Sliced sa, sb;
        slice_dense(ctx, dA.p, M, K, K, sa, SLICE_TILE_A);
        slice_dense(ctx, dB.p, N, K, K, sb, SLICE_TILE_B);
        sliced_gemm(ctx, sa, sb, dC.p, OutMap{0, N}, false);
        dC.download(C, (size_t)M * N);
        HF_CUDA(cudaStreamSynchronize(ctx.stream));
    });
}

int hfgpu_set_stream(void* stream)
{
    return guard([&] {
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        ctx.stream = stream ? (cudaStream_t)stream : ctx.own_stream;
        HF_CUBLAS(cublasSetStream(ctx.blas, ctx.stream));
        HF_CUSOLVER(cusolverDnSetStream(ctx.solver, ctx.stream));
    });
}

int hfgpu_probe_fp64_tflops(double* tflops)
{
    return guard([&] {
        check_ptr(tflops, "tflops");
        Context& ctx = context();
        std::lock_guard<std::recursive_mutex> call_lock(ctx.call_mutex);
        *tflops = probe_fp64_tflops(ctx);
    });
}

void hfgpu_default_options(hfgpu_options* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->nscf = 40;
    o->mix_alpha = 1.0;
    o->tolE = 1e-10;
    o->tolP = 1e-8;
    o->scf_accel = HFGPU_SCF_MIXING;
    o->diis_size = 8;
    o->schwarz = 0.0;
    o->mp2 = HFGPU_MP2_FP64;
    o->mp2_nocc = 0;
}

int64_t hfgpu_autotune_table(char* buf, int64_t len)
{
    const std::string s = tune_dump();
    if (buf && len > 0) {
        const int64_t k = std::min<int64_t>(len - 1, (int64_t)s.size());
        std::memcpy(buf, s.data(), (size_t)k);
        buf[k] = 0;
    }
    return (int64_t)s.size();
}

void hfgpu_autotune_clear(void) { tune_clear(); }

int hfgpu_basis_size(int natoms, const int* atno)
{
    if (natoms < 1 || !atno) return 0;
    return basis_size(natoms, atno);
}

int hfgpu_rhf(int natoms, const int* atno, const double* xyz, const hfgpu_options* opt_in, hfgpu_result* res,
              double* C, double* lam)
{
    int conv = 1, nscf = 0;
    int rc = guard([&] { rhf_impl(natoms, atno, xyz, opt_in, res, C, lam, conv, nscf); });
    if (rc == HFGPU_OK && !conv) {
        set_last_error("SCF did not converge in " + std::to_string(nscf) + " iterations.");
        return HFGPU_ERR_NOT_CONVERGED;
    }
    return rc;
}

int hfgpu_rhf_gradient(int natoms, const int* atno, const double* xyz, const hfgpu_options* opt_in,
                       hfgpu_result* res, double* grad)
{
    int conv = 1, nscf = 0;
    int rc = guard([&] {
        check_ptr(grad, "grad");
        rhf_impl(natoms, atno, xyz, opt_in, res, nullptr, nullptr, conv, nscf, grad);
    });
    if (rc == HFGPU_OK && !conv) {
        set_last_error("SCF did not converge in " + std::to_string(nscf) + " iterations.");
        return HFGPU_ERR_NOT_CONVERGED;
    }
    return rc;
}

int hfgpu_rhf_batch(int nmol, const int* natoms, const int* atno, const double* xyz, const hfgpu_options* opt,
                    hfgpu_result* res)
{
    if (nmol < 0 || (nmol > 0 && (!natoms || !atno || !xyz || !res))) {
        set_last_error("hfgpu_rhf_batch: invalid arguments");
        return HFGPU_ERR_INVALID;
    }
    std::vector<int64_t> a0(nmol + 1, 0);
    for (int m = 0; m < nmol; ++m) a0[m + 1] = a0[m] + (natoms[m] > 0 ? natoms[m] : 0);
    std::vector<int> rc(nmol, HFGPU_OK);
    std::vector<std::string> err(nmol);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        set_last_error("hfgpu_rhf_batch: no CUDA device");
        return HFGPU_ERR_NO_DEVICE;
    }
    if (!opt || opt->batch_mode == 0) {
        fused_batch(nmol, natoms, atno, xyz, a0, opt, res, rc, err, dev);
    } else {
        streams_batch(nmol, natoms, atno, xyz, a0, opt, res, rc, err, dev);
    }
    int first = HFGPU_OK;
    for (int m = 0; m < nmol; ++m)
        if (rc[m] != HFGPU_OK) {
            res[m].niter = -rc[m];
            if (first == HFGPU_OK) {
                first = rc[m];
                set_last_error("molecule " + std::to_string(m) + ": " + err[m]);
            }
        }
    return first;
}

}  // extern "C"

// hfgpu_rhf_batch, batch_mode 1: each molecule on its own context (streams, handles),
// batch_streams at once; while one waits on a host-side convergence check the
// others fill the GPU
static void streams_batch(int nmol, const int* natoms, const int* atno, const double* xyz,
                          const std::vector<int64_t>& a0, const hfgpu_options* opt, hfgpu_result* res,
                          std::vector<int>& rc, std::vector<std::string>& err, int dev)
{
    int nw = opt && opt->batch_streams > 0 ? opt->batch_streams : 8;
    nw = std::max(1, std::min(nw, std::min(nmol, 64)));
    std::atomic<int> next{0};
    auto work = [&]() {
        Context* c = nullptr;
        int r0 = guard([&] {
            HF_CUDA(cudaSetDevice(dev));
            c = context_acquire();
        });
        for (int m; (m = next.fetch_add(1)) < nmol;) {
            if (r0 != HFGPU_OK) {
                rc[m] = r0;
                err[m] = hfgpu_last_error();
                continue;
            }
            int conv = 1, nscf = 0;
            int r = guard([&] { rhf_impl(natoms[m], atno + a0[m], xyz + 3 * a0[m], opt, &res[m], nullptr, nullptr, conv,
                                         nscf, nullptr, c); });
            if (r == HFGPU_OK && !conv) {
                r = HFGPU_ERR_NOT_CONVERGED;
                set_last_error("SCF did not converge in " + std::to_string(nscf) + " iterations.");
            }
            rc[m] = r;
            if (r != HFGPU_OK) err[m] = hfgpu_last_error();
        }
        context_release(c);
    };
    if (nw == 1) {
        work();
    } else {
        std::vector<std::thread> th;
        for (int w = 0; w < nw; ++w) th.emplace_back(work);
        for (auto& t : th) t.join();
    }
}

// hfgpu_rhf_batch, batch_mode 0: waves of molecules, largest first, each wave at
// most batch_streams molecules (32 by default) whose packed integrals and MBPT2
// work arrays fit a device-memory budget; two waves in flight at a time.  One
// thread per molecule runs its pipeline; the wave's BatchWave joins their ERI
// launches and Fock builds.
static void fused_batch(int nmol, const int* natoms, const int* atno, const double* xyz,
                        const std::vector<int64_t>& a0, const hfgpu_options* opt, hfgpu_result* res,
                        std::vector<int>& rc, std::vector<std::string>& err, int dev)
{
    const int cap = opt && opt->batch_streams > 0 ? std::min(opt->batch_streams, 256) : 32;
    // sizes (molecules with bad input get 0 and fail on their own thread)
    std::vector<int> nbf(nmol, 0), order(nmol);
    for (int m = 0; m < nmol; ++m) {
        nbf[m] = natoms[m] > 0 ? hfgpu_basis_size(natoms[m], atno + a0[m]) : 0;
        order[m] = m;
    }
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return nbf[x] > nbf[y]; });
    // device bytes a molecule holds in a wave: its packed integrals and quartet
    // blocks, and at its MBPT2 stage two pair x occupied x virtual arrays
    auto bytes = [&](int m) {
        const double n = nbf[m], o = 0.2 * n, v = n - o;
        return 8.0 * (1.2 * (double)packed_size(nbf[m]) + 2.0 * n * (n + 1) / 2 * o * v + 8.0 * n * n);
    };
    size_t freeb = 0, totb = 0;
    if (cudaSetDevice(dev) != cudaSuccess || cudaMemGetInfo(&freeb, &totb) != cudaSuccess) freeb = 0;
    // two waves run at once, so that one wave's Fock builds overlap the other
    // wave's per-molecule SCF steps; each gets half of the memory budget
    constexpr int WAVES_IN_FLIGHT = 2;
    const double budget = std::max(4e9, 0.6 * (double)freeb / WAVES_IN_FLIGHT);
    std::vector<std::vector<int>> waves;
    for (size_t i = 0; i < order.size();) {
        std::vector<int> wave;
        double used = 0;
        while (i < order.size() && (int)wave.size() < cap && (wave.empty() || used + bytes(order[i]) <= budget)) {
            used += bytes(order[i]);
            wave.push_back(order[i++]);
        }
        waves.push_back(std::move(wave));
    }
    auto run_wave = [&](const std::vector<int>& wave) {
        Context* wctx = nullptr;
        const int r0 = guard([&] {
            HF_CUDA(cudaSetDevice(dev));
            wctx = context_acquire();
        });
        if (r0 != HFGPU_OK) {
            for (int m : wave) {
                rc[m] = r0;
                err[m] = hfgpu_last_error();
            }
            return;
        }
        wctx->tune = (opt && opt->autotune != 0) || tune_env_enabled();
        {
            BatchWave bw((int)wave.size(), wctx);
            auto work = [&](int k) {
                const int m = wave[k];
                BatchMember mem{&bw, k};
                Context* c = nullptr;
                int r = guard([&] {
                    HF_CUDA(cudaSetDevice(dev));
                    c = context_acquire();
                });
                int conv = 1, nscf = 0;
                if (r == HFGPU_OK)
                    r = guard([&] { rhf_impl(natoms[m], atno + a0[m], xyz + 3 * a0[m], opt, &res[m], nullptr, nullptr,
                                             conv, nscf, nullptr, c, &mem); });
                else
                    bw.leave(k);
                if (r == HFGPU_OK && !conv) {
                    r = HFGPU_ERR_NOT_CONVERGED;
                    set_last_error("SCF did not converge in " + std::to_string(nscf) + " iterations.");
                }
                rc[m] = r;
                if (r != HFGPU_OK) err[m] = hfgpu_last_error();
                context_release(c);
            };
            std::vector<std::thread> th;
            for (size_t k = 0; k < wave.size(); ++k) th.emplace_back(work, (int)k);
            for (auto& t : th) t.join();
        }
        context_release(wctx);
    };
    std::atomic<size_t> next{0};
    auto wave_worker = [&]() {
        for (size_t w; (w = next.fetch_add(1)) < waves.size();) run_wave(waves[w]);
    };
    const int nthreads = (int)std::min<size_t>(WAVES_IN_FLIGHT, waves.size());
    if (nthreads <= 1) {
        wave_worker();
    } else {
        std::vector<std::thread> wt;
        for (int t = 0; t < nthreads; ++t) wt.emplace_back(wave_worker);
        for (auto& t : wt) t.join();
    }
}
