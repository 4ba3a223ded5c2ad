// Device-side integral plan of one molecule: basis, shell pairs with their
// primitive-pair records, Schwarz bounds and the screened quartet segments of
// every class.  Shared by the ERI, Fock-digest and gradient translation units.
#pragma once
#include <memory>
#include <vector>

#include "eri_kernel.cuh"
#include "internal.h"

namespace hfgpu {

struct ClassPlan {
    int tb, tk;
    std::vector<Seg> segs;
    std::vector<int64_t> kprod;  // primitive quartets per quartet, per segment
    int lane_target = 16;        // primitive quartets per lane that the splits were laid out for
    int64_t nwarps = 0;
    int64_t nq = 0;     // quartets of the class
    int64_t boff = 0;   // offset of the class's blocks in EriPlan::blocks
    int64_t qbase = 0;  // offset of the class's quartets in EriPlan::qlist
    DBuf<Seg> dsegs;
};

struct EriPlan {
    Basis basis;
    int npair = 0;
    // device basis
    DBuf<int> sL, snp, sp0, sc0, scf, cfn;
    DBuf<double> sxyz, alpha, coef;
    // pairs
    std::vector<int> pA, pB, pK, pT;
    std::vector<int64_t> poff;
    DBuf<int> dA, dB, dK;
    DBuf<int64_t> doff;
    DBuf<double> pdata;
    // screening
    std::vector<double> Q;
    DBuf<double> dQ;
    DBuf<int> gpairs;
    DBuf<int64_t> prefix;
    std::vector<ClassPlan> classes;
    DBuf<double> blocks;  // class-wise quartet blocks, kept for the SCF's Fock builds
    DBuf<int2> qlist;     // (bra, ket) pair ids of every kept quartet, class by class
    DBuf<int> pair_mol;   // batched plans: the molecule of every pair
    EriStats stats;
    // around the ERI pass (eri_compute_start / _finish): ev0 on the main stream
    // before it, ev_end[i] after the last class launched on side stream i
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_end[8] = {};
    int n_ev_end = 0;
    // host copies of the grouped pair ids and prefix sums (for merging plans)
    std::vector<int> h_gpairs;
    std::vector<int64_t> h_prefix;
    // batched plans (eri_plan_merge): the molecules' basis sizes, shell counts and
    // first shells, and each molecule's packed-array offset in the output of
    // eri_compute (device; null for one molecule)
    int nmol = 1;
    std::vector<int> mol_nbf, mol_ns, mol_sh0;
    DBuf<int64_t> mol_out;

    EriPlan() = default;
    EriPlan(const EriPlan&) = delete;
    EriPlan& operator=(const EriPlan&) = delete;
    ~EriPlan()
    {
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        for (auto e : ev_end)
            if (e) cudaEventDestroy(e);
    }

    ShellDev shdev() const
    {
        return ShellDev{sL.p, snp.p, sxyz.p, sp0.p, sc0.p, scf.p, alpha.p, coef.p, cfn.p};
    }
    PairDev prdev() const { return PairDev{dA.p, dB.p, dK.p, doff.p, pdata.p}; }
};

}  // namespace hfgpu
