// Generalized symmetric-definite eigensolver F C = S C diag(lam) (eigh.cu).
#pragma once
#include "internal.h"

namespace hfgpu {

struct TrdSync {
    unsigned count, gen;
    int err, pad;
};

// X = L^-T from the Cholesky factor S = L L^T, so that X^T S X = I (n x n, column-major)
void cholesky_orthogonalizer(Context& ctx, int n, const double* dS, double* dX);

// eigenvalues (ascending) and eigenvectors of the symmetric tridiagonal matrix
// with diagonal d and off-diagonal e; Z (n x ncol, column-major) gets the
// eigenvectors of the ncol lowest eigenvalues (tridiag.cpp)
void tridiag_eigen(int n, const double* d, const double* e, double* lam, double* Z, int ncol);

// F C = S C diag(lam), given the orthogonaliser X of S:
//   F' = X^T F X, Householder tridiagonalisation Q^T F' Q = T on the GPU (one
//   cooperative kernel), T = Z diag(lam) Z^T on the host, C = X Q Z by GEMMs.
// F must be symmetric (both triangles); C may alias F.  Work buffers live as long
// as the object, so an SCF reuses them every iteration.
struct Eigh {
    int n = 0;
    DBuf<double> Fp, T1, V, tau, de, xch, Tinv, Tw, XV, M, W;
    DBuf<TrdSync> sync;
    double* hbuf = nullptr;  // pinned: d, e (2n), lam (n), Z (n x n), barrier state
    cudaEvent_t ready = nullptr;
    static bool supported(Context& ctx, int n);
    void setup(Context& ctx, int n_);
    // ncol: eigenvectors formed (the lowest ncol; all eigenvalues always); <= 0: all
    void solve(Context& ctx, const double* X, const double* F, double* C, double* lam, int ncol = 0);
    ~Eigh();
};

// the drop-in eigh: A (lower triangle used) C = B C diag(lam), B positive
// definite; solver 0 = own where supported, else (or 1) cuSOLVER dsygvd
void eigh_generalized(Context& ctx, int n, const double* dA, const double* dB, double* dC, double* dLam, int solver);

}  // namespace hfgpu
