// BatchWave (batch.h): the rendezvous of a wave's molecules at their shared
// ERI pass and at every batched Fock build.
#include <numeric>

#include "batch.h"
#include "eri_plan.h"

namespace hfgpu {

BatchWave::BatchWave(int nmol, Context* ctx)
    : nmol_(nmol), ctx_(ctx), state_(nmol, 0), plans_(nmol, nullptr), ev_(nmol, nullptr), requested_(nmol, 0),
      reqP_(nmol, nullptr), reqG_(nmol, nullptr), reqScreen_(nmol, 0.0), mol_off_(nmol, 0), mol_flops_(nmol, 0.0)
{
    for (int m = 0; m < nmol; ++m) HF_CUDA(cudaEventCreateWithFlags(&ev_[m], cudaEventDisableTiming));
    HF_CUDA(cudaEventCreateWithFlags(&done_, cudaEventDisableTiming));
    HF_CUDA(cudaEventCreate(&t0_));
    HF_CUDA(cudaEventCreate(&t1_));
}

BatchWave::~BatchWave()
{
    if (ctx_) cudaStreamSynchronize(ctx_->stream);
    delete merged_;
    for (auto e : ev_)
        if (e) cudaEventDestroy(e);
    if (done_) cudaEventDestroy(done_);
    if (t0_) cudaEventDestroy(t0_);
    if (t1_) cudaEventDestroy(t1_);
}

void BatchWave::fail_locked(const std::exception_ptr& e)
{
    if (!failure_) failure_ = e;
    cv_.notify_all();
}

// every molecule that reached the ERIs has its plan: merge, allocate each
// molecule's packed array and the shared quartet blocks, one launch per class
void BatchWave::run_eri_locked()
{
    try {
        cudaStream_t st = ctx_->stream;
        std::vector<EriPlan*> live;
        std::vector<int> slot(nmol_, -1);
        for (int m = 0; m < nmol_; ++m)
            if (state_[m] == 1) {
                HF_CUDA(cudaStreamWaitEvent(st, ev_[m], 0));
                slot[m] = (int)live.size();
                live.push_back(plans_[m]);
            }
        merged_ = eri_plan_merge(*ctx_, live);
        // packed arrays of the molecules in the merged plan's order
        std::vector<int64_t> offs(live.size(), 0);
        int64_t total = 0;
        for (size_t i = 0; i < live.size(); ++i) {
            offs[i] = total;
            total += packed_size(live[i]->basis.nbf);
        }
        packed_.alloc(std::max<int64_t>(total, 1), st);
        packed_.zero();
        merged_->mol_out = to_device(offs, st);
        for (int m = 0; m < nmol_; ++m)
            if (slot[m] >= 0) {
                mol_off_[m] = offs[slot[m]];
                mol_flops_[m] = plans_[m]->stats.flops;
            }
        EriStats es;
        eri_compute(*ctx_, merged_, packed_.p, true, &es);
        eri_ms_ = es.ms;
        tables_.setup(*ctx_, merged_, st);
        HF_CUDA(cudaEventRecord(done_, st));
        HF_CUDA(cudaEventSynchronize(done_));
        // the digest tables address molecules by their place in the merged plan
        slot_ = slot;
    } catch (...) {
        fail_locked(std::current_exception());
    }
    ++eri_done_;
    cv_.notify_all();
}

double* BatchWave::eri_rendezvous(int mol, Context& c, EriPlan* plan, double* ms_eri)
{
    std::unique_lock<std::mutex> lk(mu_);
    HF_CHECK(state_[mol] == 0, HFGPU_ERR_INVALID, "batch: molecule arrived twice");
    plans_[mol] = plan;
    HF_CUDA(cudaEventRecord(ev_[mol], c.stream));
    state_[mol] = 1;
    ++arrived_;
    ++active_;
    if (arrived_ + left_early_ == nmol_) run_eri_locked();
    cv_.wait(lk, [&] { return eri_done_ > 0 || failure_; });
    if (failure_) std::rethrow_exception(failure_);
    HF_CUDA(cudaStreamWaitEvent(c.stream, done_, 0));
    // this molecule's share of the batched ERI time, by its McMurchie-Davidson flops
    double tot = 0;
    for (double f : mol_flops_) tot += f;
    if (ms_eri) *ms_eri = tot > 0 ? eri_ms_ * mol_flops_[mol] / tot : 0.0;
    return packed_.p + mol_off_[mol];
}

void BatchWave::run_digest_locked()
{
    try {
        cudaStream_t st = ctx_->stream;
        // the tables of the previous build must have been copied before they change
        HF_CUDA(cudaEventSynchronize(done_));
        tables_.wait_tables();
        for (int m = 0; m < nmol_; ++m) {
            const int s = slot_[m];
            if (s < 0) continue;
            if (requested_[m]) {
                HF_CUDA(cudaStreamWaitEvent(st, ev_[m], 0));
                tables_.h_P[s] = reqP_[m];
                tables_.h_G[s] = reqG_[m];
                tables_.h_screen[s] = reqScreen_[m];
            } else {
                tables_.h_screen[s] = -1.0;
            }
        }
        HF_CUDA(cudaEventRecord(t0_, st));
        eri_digest_batch(*ctx_, merged_, tables_, st);
        HF_CUDA(cudaEventRecord(t1_, st));
        HF_CUDA(cudaEventRecord(done_, st));
        ++builds_;
        pending_timer_ = true;
    } catch (...) {
        fail_locked(std::current_exception());
    }
    std::fill(requested_.begin(), requested_.end(), 0);
    pending_ = 0;
    ++round_;
    cv_.notify_all();
}

void BatchWave::digest(int mol, Context& c, const double* P, double* G, double screen)
{
    std::unique_lock<std::mutex> lk(mu_);
    if (failure_) std::rethrow_exception(failure_);
    HF_CHECK(state_[mol] == 1, HFGPU_ERR_INVALID, "batch: Fock build for a molecule outside the wave");
    if (pending_timer_) {  // time the previous build (it has finished: this molecule waited on it)
        float ms = 0;
        if (cudaEventElapsedTime(&ms, t0_, t1_) == cudaSuccess) fock_ms_ += ms;
        pending_timer_ = false;
    }
    HF_CUDA(cudaEventRecord(ev_[mol], c.stream));
    reqP_[mol] = P;
    reqG_[mol] = G;
    reqScreen_[mol] = screen > 0 ? screen : 0.0;
    requested_[mol] = 1;
    ++pending_;
    const int64_t my = round_;
    if (pending_ == active_) run_digest_locked();
    cv_.wait(lk, [&] { return round_ > my || failure_; });
    if (failure_) std::rethrow_exception(failure_);
    HF_CUDA(cudaStreamWaitEvent(c.stream, done_, 0));
}

void BatchWave::leave(int mol)
{
    std::unique_lock<std::mutex> lk(mu_);
    if (state_[mol] == 2) return;
    if (state_[mol] == 0) {
        state_[mol] = 2;
        ++left_early_;
        if (eri_done_ == 0 && arrived_ > 0 && arrived_ + left_early_ == nmol_) run_eri_locked();
        else if (arrived_ == 0 && left_early_ == nmol_) cv_.notify_all();
        return;
    }
    state_[mol] = 2;
    --active_;
    if (requested_[mol]) {  // cannot happen: a molecule leaves between builds
        requested_[mol] = 0;
        --pending_;
    }
    if (pending_ > 0 && pending_ == active_) run_digest_locked();
}

}  // namespace hfgpu
