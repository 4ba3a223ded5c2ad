// A wave of molecules that share their integral and Fock-build launches.
//
// Each molecule of a wave runs the rhf_gauss pipeline (src/drivers.f90:12-51)
// on its own worker thread and context.  Its quartet plan is handed to the wave
// (eri_rendezvous); when every molecule has one, the plans are merged and one
// launch per quartet class computes all their integrals (packed arrays and
// quartet blocks).  Every SCF iteration each molecule asks for G(P)
// (digest): when every molecule still iterating has asked, one batched Fock
// build (a CUDA graph of one launch per class) serves all of them.  A
// converged or failed molecule leaves, and the next builds go on without it.
// The per-molecule steps between builds (F, DIIS, density, convergence) run
// on each molecule's own streams.
#pragma once
#include <condition_variable>
#include <exception>
#include <memory>
#include <mutex>
#include <vector>

#include "internal.h"

namespace hfgpu {

class BatchWave {
public:
    BatchWave(int nmol, Context* ctx);
    ~BatchWave();
    // molecule mol's plan (made on context c, whose stream orders it); returns
    // the device address of its packed integrals once the wave's ERIs are done
    // (c's stream waits for them) and its share of the ERI time
    double* eri_rendezvous(int mol, Context& c, EriPlan* plan, double* ms_eri);
    // G = J - K/2 of P into G (device, molecule mol's n x n), screened at
    // screen (0: full build), in stream order on c's stream
    void digest(int mol, Context& c, const double* P, double* G, double screen);
    // mol takes no further part (converged, failed, or never reached the ERIs)
    void leave(int mol);
    double fock_ms() const { return fock_ms_; }
    int builds() const { return builds_; }

private:
    void run_eri_locked();
    void run_digest_locked();
    void fail_locked(const std::exception_ptr& e);
    std::mutex mu_;
    std::condition_variable cv_;
    int nmol_;
    Context* ctx_;  // the wave's own context (stream) for the shared launches
    std::vector<int> state_;  // 0: before the ERIs, 1: iterating, 2: left
    int arrived_ = 0, left_early_ = 0, active_ = 0, pending_ = 0;
    int64_t eri_done_ = 0, round_ = 0;
    std::vector<EriPlan*> plans_;
    std::vector<cudaEvent_t> ev_;  // per molecule, recorded on its stream at its request
    std::vector<char> requested_;
    std::vector<const double*> reqP_;
    std::vector<double*> reqG_;
    std::vector<double> reqScreen_;
    EriPlan* merged_ = nullptr;
    DBuf<double> packed_;
    std::vector<int64_t> mol_off_;
    std::vector<int> slot_;  // each molecule's place in the merged plan (-1: not in it)
    bool pending_timer_ = false;
    std::vector<double> mol_flops_;
    double eri_ms_ = 0, fock_ms_ = 0;
    int builds_ = 0;
    BatchDigest tables_;
    cudaEvent_t done_ = nullptr, t0_ = nullptr, t1_ = nullptr;
    std::exception_ptr failure_;
};

}  // namespace hfgpu
