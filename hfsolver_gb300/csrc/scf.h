// SCF driver interface (scf.cu) and the MP2 stage (mp2.cu).
#pragma once
#include "internal.h"

namespace hfgpu {

// G = J - K/2 of the density dP into dG.  screen > 0: a density difference;
// quartets whose Schwarz bound times the largest |dP| element they touch is
// below screen may be left out.
using DirectJK = void (*)(Context& ctx, void* user, const double* dP, double* dG, double screen);

struct ScfIn {
    int n = 0, nocc = 0, nscf = 40;
    const double* dH = nullptr;
    const double* dS = nullptr;
    const double* d_int2 = nullptr;  // packed integrals (in-core Fock build)
    DirectJK direct_jk = nullptr;    // or: integral-direct Fock build
    void* direct_ctx = nullptr;
    double tolE = 1e-10, tolP = 1e-8, alpha = 1.0;
    int accel = HFGPU_SCF_MIXING;
    int diis_size = 8;
    bool purify = false;  // density by SP2 purification instead of dsygvd each iteration
    // incremental Fock builds (direct_jk only): G(P_k) = G(P_j) + G(P_k - P_j)
    // with the difference screened at inc_screen; a full build every
    // inc_rebuild iterations and before convergence is accepted.  0: off.
    double inc_screen = 0.0;
    int inc_rebuild = 8;
    // starting density (device, n x n); null: P = 0 as in the reference's doscf
    const double* dP0 = nullptr;
    // eigensolver: 0 = own (eigh.cu: GPU tridiagonalisation, host tridiagonal
    // solve) where it fits (3 <= n <= 1024), else cuSOLVER dsygvd; 1 = dsygvd
    int eigensolver = 0;
    // optional: called first (before the SCF's own set-up is queued) and right
    // before the first Fock build, so that work started by `begin` on side
    // streams (the ERI pass) runs under the set-up; `end` joins it
    void (*begin)(void* user) = nullptr;
    void (*end)(void* user) = nullptr;
    void* hook_user = nullptr;
};

struct ScfOut {
    double E0 = 0, dP = 0;
    int niter = 0;
    bool converged = false;
};

ScfOut run_scf(Context& ctx, const ScfIn& in, double* dC, double* dP, double* dLam);
double device_dot(Context& ctx, int64_t nn, const double* A, const double* B);

// (i a | j b) for i, j over the n1 columns of C1 and a, b over the n2 columns
// of C2 (both n x n1 / n x n2, column-major, leading dimension n), from the
// packed AO integrals.  Output layout [i][a][j][b].
void ao2mo_fp64(Context& ctx, int n, const double* d_int2, const double* dC1, int n1, const double* dC2, int n2,
                double* d_out);
// C[m][n] = alpha A[m][k] B[k][n] + beta C, row-major FP64 with leading
// dimensions lda, ldb, ldc: the row-gathered FP64 GEMM of dgemm_rows.cu
void dgemm_rowmajor(Context& ctx, int64_t m, int n, int k, double alpha, const double* A, int64_t lda,
                    const double* B, int64_t ldb, double beta, double* C, int64_t ldc);
// E2 from (ia|jb) in [i][a][j][b] layout and orbital energies (device)
double mp2_energy(Context& ctx, int nocc, int nvir, const double* d_iajb, const double* d_eps);

}  // namespace hfgpu

namespace hfgpu {
// full (ij|kl) over all orbitals into the packed layout (transform_int2 drop-in)
void transform_packed(Context& ctx, int n, const double* d_int2, const double* dC, double* d_mo);
// MBPT2 energy with the tensor-core (exactly sliced bf16) transform (mp2_mixed.cu)
double mp2_energy_mixed(Context& ctx, int n, const double* d_int2, const double* dC, int nocc, const double* d_eps);
// Green's-function pole of orbital i (0-based) by find_pole_diag's fixed-point
// iteration (gf.cu); HFGPU_ERR_NOT_CONVERGED after nscf iterations
double find_pole_diag(Context& ctx, int n, const double* d_mo, const double* d_lam, int nocc, int i, int nscf,
                      double tolE, int* niter);
// term1 of src/mbpt2.f90 on packed MO integrals (mbpt2 drop-in)
double mbpt2_packed(Context& ctx, int n, const double* d_mo, const double* d_lam, int nocc);
// E3 of src/mbpt3.f90 on packed MO integrals (mbpt3 drop-in, mbpt3.cu)
double mbpt3_packed(Context& ctx, int n, const double* d_mo, const double* d_lam, int nocc);
}  // namespace hfgpu
