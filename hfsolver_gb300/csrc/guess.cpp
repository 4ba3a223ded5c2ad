// Starting density for hfgpu_rhf: superposition of atomic densities (SAD).
//
// The reference's doscf starts from P = 0 (src/scf.f90:72-107), i.e. its first
// Fock matrix is the core Hamiltonian; the drop-in hfgpu_doscf keeps that.  The
// pipeline entry point may start closer to the answer: the molecule's density
// is guessed as the block-diagonal sum of free-atom densities in the same basis,
// each from a small closed-shell SCF of the atom (or of its cation with one
// electron fewer for odd Z, scaled back to Z electrons; for hydrogen, the lowest
// orbital of the one-electron Hamiltonian).  The p-p blocks are averaged over
// the three directions (a closed-shell open-p atom would otherwise fix an
// arbitrary axis) and the s-p, p-d cross blocks, which vanish for a spherical
// atom, are dropped.  Atomic densities are computed once per element and cached.
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "internal.h"
#include "md.cuh"
#include "scf.h"

namespace hfgpu {

namespace {
std::mutex g_sad_mutex;
std::map<int, std::vector<double>> g_sad;  // Z -> atomic density, nZ x nZ column-major
}  // namespace

static std::vector<double> atom_density(Context& ctx, int Z)
{
    const double xyz[3] = {0.0, 0.0, 0.0};
    Basis b = build_basis(1, &Z, xyz);
    const int n = b.nbf;
    const size_t nn = (size_t)n * n;
    cudaStream_t st = ctx.stream;
    DBuf<double> dS(nn, st), dT(nn, st), dV(nn, st), dH(nn, st);
    const double zero = 0.0;
    onee_compute(ctx, b, 1, &Z, &zero, &zero, &zero, dS.p, dT.p, dV.p);
    const double one = 1.0;
    HF_CUBLAS(cublasDgeam(ctx.blas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, &one, dT.p, n, &one, dV.p, n, dH.p, n));
    DBuf<double> dI(packed_size(n), st);
    dI.zero();
    std::unique_ptr<EriPlan, void (*)(EriPlan*)> plan(eri_plan_create(ctx, b, 0.0), eri_plan_destroy);
    eri_compute_packed(ctx, plan.get(), dI.p, nullptr);
    const int nel = (Z % 2 == 0 || Z == 1) ? Z : Z - 1;  // closed shell: the atom, or its cation
    ScfIn in;
    in.n = n;
    in.nocc = Z == 1 ? 0 : nel / 2;
    in.nscf = 100;
    in.dH = dH.p;
    in.dS = dS.p;
    in.d_int2 = dI.p;
    in.tolE = 1e-8;
    in.tolP = 1e-6;
    in.accel = HFGPU_SCF_DIIS;
    DBuf<double> dC(nn, st), dP(nn, st), dL(n, st);
    run_scf(ctx, in, dC.p, dP.p, dL.p);  // an unconverged atom is still a usable guess
    std::vector<double> P(nn), C(nn);
    dP.download(P.data(), nn);
    dC.download(C.data(), nn);
    HF_CUDA(cudaStreamSynchronize(st));
    if (Z == 1) {  // one electron in the lowest orbital of H
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) P[i + (size_t)j * n] = C[i] * C[j];
    } else if (nel != Z) {
        for (double& v : P) v *= (double)Z / nel;
    }
    // spherical average: p-p blocks -> (trace / 3) I; s-p and p-d blocks -> 0
    std::vector<int> first, L;
    int f = 0;
    for (auto& sh : b.shells) {
        first.push_back(f);
        L.push_back(sh.L);
        f += ncart(sh.L);
    }
    for (size_t a = 0; a < b.shells.size(); ++a)
        for (size_t c = 0; c < b.shells.size(); ++c) {
            const int fa = first[a], fc = first[c], na = ncart(L[a]), nc = ncart(L[c]);
            auto at = [&](int i, int j) -> double& { return P[(size_t)(fa + i) + (size_t)(fc + j) * n]; };
            if (L[a] == 1 && L[c] == 1) {
                const double tr = (at(0, 0) + at(1, 1) + at(2, 2)) / 3.0;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) at(i, j) = i == j ? tr : 0.0;
            } else if ((L[a] == 1) != (L[c] == 1)) {
                for (int i = 0; i < na; ++i)
                    for (int j = 0; j < nc; ++j) at(i, j) = 0.0;
            }
        }
    return P;
}

void sad_guess(Context& ctx, int natoms, const int* atno, int nbf, double* dP0)
{
    std::vector<double> P((size_t)nbf * nbf, 0.0);
    int off = 0;
    for (int a = 0; a < natoms; ++a) {
        const int Z = atno[a];
        std::vector<double> Pa;
        {
            std::lock_guard<std::mutex> lk(g_sad_mutex);
            auto it = g_sad.find(Z);
            if (it != g_sad.end()) Pa = it->second;
        }
        if (Pa.empty()) {
            Pa = atom_density(ctx, Z);
            std::lock_guard<std::mutex> lk(g_sad_mutex);
            g_sad[Z] = Pa;
        }
        const int na = (int)std::lround(std::sqrt((double)Pa.size()));
        HF_CHECK(off + na <= nbf, HFGPU_ERR_INVALID, "atomic guess does not fit the basis");
        for (int j = 0; j < na; ++j)
            for (int i = 0; i < na; ++i) P[(size_t)(off + i) + (size_t)(off + j) * nbf] = Pa[(size_t)i + (size_t)j * na];
        off += na;
    }
    HF_CHECK(off == nbf, HFGPU_ERR_INVALID, "atomic guess does not cover the basis");
    HF_CUDA(cudaMemcpyAsync(dP0, P.data(), sizeof(double) * P.size(), cudaMemcpyHostToDevice, ctx.stream));
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
}

}  // namespace hfgpu
