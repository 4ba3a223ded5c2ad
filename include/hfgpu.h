/*
 * hfgpu — GB300-native (sm_103a) kernels for hfsolver's molecular
 * Gaussian-orbital path: contracted electron-repulsion integrals, the RHF Fock
 * build, the AO->MO transform and the MBPT2 energy.
 *
 * C ABI.  Plain pointers and sizes; every entry point returns an int status
 * (HFGPU_OK = 0) instead of aborting the process the way the reference's
 * stop_error does, and hfgpu_last_error() gives the message of the last
 * failure on the calling thread.  All arrays are host memory owned by the
 * caller, as in the reference (the callee only writes outputs); device memory
 * is managed inside the library on the current CUDA device, and each call
 * returns after its results are in the caller's buffers.
 *
 * Matrices are column-major n x n, like the Fortran arrays they replace.
 * Packed two-electron arrays use hfsolver's 8-fold index
 * (src/cints.c:327-347 and src/scf.f90:184-223) with 64-bit positions:
 * (ij|kl) with i>=j, k>=l, ij>=kl, ij = i(i+1)/2+j, lives at ij(ij+1)/2+kl
 * (0-based); its length is m(m+1)/2 with m = n(n+1)/2.
 */
#ifndef HFGPU_H
#define HFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    HFGPU_OK = 0,
    HFGPU_ERR_INVALID = 1,        /* bad argument: sizes, NaN coordinates, unknown Z */
    HFGPU_ERR_CUDA = 2,           /* CUDA, cuBLAS or cuSOLVER failure */
    HFGPU_ERR_NOT_CONVERGED = 3,  /* SCF did not converge in nscf iterations */
    HFGPU_ERR_LINALG = 4,         /* eigensolver failure (S not positive definite) */
    HFGPU_ERR_UNSUPPORTED = 5,    /* angular momentum beyond d, or similar */
    HFGPU_ERR_NOMEM = 6,          /* device memory exhausted */
    HFGPU_ERR_NO_DEVICE = 7       /* no CUDA device */
};

const char *hfgpu_last_error(void);
int hfgpu_version(void);

/* Run subsequent calls on the current device on the given cudaStream_t (NULL:
 * the library's own stream); calls stay synchronous with respect to the host. */
int hfgpu_set_stream(void *cuda_stream);
/* number of libhfgpu kernels launched by this process so far (CUDA library
 * kernels such as cuBLAS/cuSOLVER are not counted) */
int64_t hfgpu_kernel_launches(void);
/* Measured FP64 FMA throughput of the current GPU in TFLOP/s (a register-only
 * kernel of independent fma chains over all SMs), the denominator used for
 * the FP64-bound integral kernels' roofline. */
int hfgpu_probe_fp64_tflops(double *tflops);

/* ---- Integral drivers: same arguments as hfsolver's C drivers --------------
 * nbf functions; function i has nprim[i] primitives starting at the 0-based
 * offset istart[i] in coef/alpha (n2 entries), centre (xcenter[i], ycenter[i],
 * zcenter[i]) and Cartesian powers (lpower[i], mpower[i], npower[i]); coef
 * already includes primitive and contraction normalisation. */

/* replaces getS, src/qc.h:8-12 / src/qc.c:6-31 (S column-major nbf x nbf) */
int hfgpu_getS(int nbf, const int *nprim, const int *istart, const double *xcenter,
               const double *ycenter, const double *zcenter, const int *lpower, const int *mpower,
               const int *npower, int n2, const double *coef, const double *alpha, double *S);

/* replaces getT, src/qc.h:14-18 / src/qc.c:33-58 */
int hfgpu_getT(int nbf, const int *nprim, const int *istart, const double *xcenter,
               const double *ycenter, const double *zcenter, const int *lpower, const int *mpower,
               const int *npower, int n2, const double *coef, const double *alpha, double *T);

/* replaces getV, src/qc.h:20-25 / src/qc.c:61-93 (nat nuclei of charge atno at x, y, z) */
int hfgpu_getV(int nbf, const int *nprim, const int *istart, const double *xcenter,
               const double *ycenter, const double *zcenter, const int *lpower, const int *mpower,
               const int *npower, int n2, const double *coef, const double *alpha, int nat,
               const int *atno, const double *x, const double *y, const double *z, double *V);

/* replaces getInts, src/qc.h:27-31 / src/qc.c:95-131: every unique (ij|kl) into
 * the packed array Ints (length m(m+1)/2, 64-bit positions).  No screening:
 * every quartet is computed, as in the reference. */
int hfgpu_getInts(int nbf, const int *nprim, const int *istart, const double *xcenter,
                  const double *ycenter, const double *zcenter, const int *lpower,
                  const int *mpower, const int *npower, int n2, const double *coef,
                  const double *alpha, double *Ints);

/* replaces the plugin routine getints2 of module gaussians,
 * src/gaussians_hfsolver.f90:13-34 (called from src/basis.f90:567): Fortran
 * layout center(3,n), power(3,n), 1-based istart; nint2 is the length of int2
 * and must equal m(m+1)/2. */
int hfgpu_getints2(int n, const int *nprim, const int *istart, const double *center,
                   const int *power, int n2, const double *coef, const double *alpha,
                   double *int2, int64_t nint2);

/* ---- SCF, transform, MBPT2 ------------------------------------------------ */

/* replaces doscf, src/scf.f90:72-136: P = 0 start, F = H + G(P) with
 * G(i,j) = sum_kl P(k,l) [(ij|kl) - (il|kj)/2] from the packed int2, generalised
 * eigenproblem F C = S C lam, P = 2 C_occ C_occ^T, convergence when
 * sqrt(sum (P - Pold)^2 / 4) < tolP and the last four energies span < tolE
 * (checked from iteration 4), else linear mixing P = (1-alpha) Pold + alpha P.
 * Outputs C (n x n), P (n x n), lam (n), E0 (electronic energy of the last
 * iteration) and the iteration count; HFGPU_ERR_NOT_CONVERGED after nscf. */
int hfgpu_doscf(int n, const double *H, const double *int2, const double *S, int nocc, int nscf,
                double tolE, double tolP, double alpha, double *C, double *P, double *lam,
                double *E0, int *niter);

/* Coulomb and exchange matrices of a density, J(i,j) = sum_kl (ij|kl) P(k,l) and
 * K(i,j) = sum_kl (ik|jl) P(k,l) (the two parts of TT, src/scf.f90:84-105), for a
 * basis in the C-driver layout above, with quartets whose Schwarz bound
 * sqrt((ab|ab)(cd|cd)) is below schwarz left out (0: none).  The integrals are
 * built and digested on the device; no two-electron array is returned. */
int hfgpu_jk(int nbf, const int *nprim, const int *istart, const double *xcenter,
             const double *ycenter, const double *zcenter, const int *lpower, const int *mpower,
             const int *npower, int n2, const double *coef, const double *alpha, const double *P,
             double schwarz, double *J, double *K);

/* replaces eigh (deigh_generalized, src/linalg.f90:241-275, LAPACK dsygvd): all
 * eigenvalues lam (ascending) and eigenvectors C (column-major, C^T B C = I) of
 * A C = B C diag(lam), A symmetric and B symmetric positive definite, both n x n
 * column-major with only their lower triangles read.  The GPU tridiagonalises
 * X^T A X (X = L^-T, B = L L^T) in one cooperative kernel and the host solves the
 * tridiagonal problem; cuSOLVER dsygvd for n < 3 or n > 1024. */
int hfgpu_eigh(int n, const double *A, const double *B, double *lam, double *C);

/* the algorithmic FP64 flop count of one primitive shell quartet of angular momenta
 * (la lb | lc ld) used for the ERI roofline (McMurchie-Davidson count,
 * hfsolver_gb300/roofline.py states the same formula); host only */
double hfgpu_md_flops(int la, int lb, int lc, int ld);

/* the host half of hfgpu_eigh: eigenvalues lam (ascending) and orthonormal
 * eigenvectors Z (n x n, column-major) of the symmetric tridiagonal matrix with
 * diagonal d (n) and off-diagonal e (n - 1).  Implicit QL for the eigenvalues,
 * inverse iteration with reorthogonalisation inside clusters for the vectors.
 * Host memory only; needs no GPU. */
int hfgpu_tridiag_eigen(int n, const double *d, const double *e, double *lam, double *Z);

/* replaces formG / formG2, src/scf.f90:26-58: G(i,j) = sum_kl P(k,l) [(ij|kl) - (il|kj)/2]
 * from the packed integrals, without the reference's dense TT(n,n,n,n)
 * (src/scf.f90:79-105); P and G column-major n x n.  P must be symmetric (a
 * density always is): the kernel reads both triangles and folds the
 * permutational copies of each integral assuming P(k,l) = P(l,k). */
int hfgpu_formG(int n, const double *P, const double *int2, double *G);

/* Allocation-free variant of hfgpu_formG; it has no counterpart in the
 * reference.  For callers that cannot let a library allocate device memory:
 * code whose device memory is all owned by its own allocator (for example a
 * framework's caching allocator that has reserved the GPU) or by a fixed
 * quota, or a latency-critical loop where a cudaMalloc would synchronise the
 * device.  Inputs and output are DEVICE pointers owned by the caller:
 * d_int2 (packed, m(m+1)/2 doubles), d_P and d_G (n x n, column-major; P
 * symmetric, as for hfgpu_formG).  The work is enqueued on cuda_stream (a
 * cudaStream_t; NULL = the legacy default stream) and the call returns without
 * waiting for it.  The only scratch is a fixed array of 512 x 512 doubles
 * (2 MiB) per device, kept until the process exits, so n <= 512 (larger n
 * returns HFGPU_ERR_INVALID).  That array's memory is taken when the library's
 * module is loaded on the device: by any libhfgpu call that sets up the
 * library on that device, or else by the first call of this function there,
 * which also looks up the array's device address.  Make that first call before
 * reserving the device's memory (HFGPU_ERR_NOMEM otherwise) and before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * race.  An error already pending in the CUDA runtime when the call starts is
 * returned as HFGPU_ERR_CUDA without launching anything.  Calls must not cross
 * a cudaDeviceReset (the cached address belongs to the device's context). */
int hfgpu_formG_device_noalloc(int n, const double *d_int2, const double *d_P, double *d_G, void *cuda_stream);

/* replaces transform_int2, src/mbpt.f90:11-79: (mu nu|la si) -> (ij|kl) over
 * all orbitals, both arrays packed.  FP64. */
int hfgpu_transform_int2(int n, const double *int2, const double *C, double *moint2);

/* replaces mbpt2, src/mbpt.f90:154-159 (term1, src/mbpt2.f90:8-31):
 * E2 = sum_{a,b<nocc; r,s>=nocc} [2 (ar|bs)^2 - (ar|bs)(as|br)] / (lam_a+lam_b-lam_r-lam_s)
 * from the packed MO integrals. */
int hfgpu_mbpt2(int n, const double *moint2, const double *lam, int nocc, double *E2);

/* replaces mbpt3, src/mbpt.f90:161-169 (term1 + term2 + term3 of
 * src/mbpt3.f90:8-128): the third-order energy from the packed MO integrals,
 * all electrons correlated.  FP64; the terms run as dense GEMMs over compound
 * occupied-virtual indices (the project's FP64 GEMM kernels) instead of the
 * reference's six nested loops. */
int hfgpu_mbpt3(int n, const double *moint2, const double *lam, int nocc, double *E3);

/* replaces find_pole_diag, src/gf.f90:15-34: the Green's-function pole of
 * orbital i (1-based, as the Fortran function takes it) by the fixed-point
 * iteration E <- lam(i) + Sigma_ii(E) from E = lam(i), with the second-order
 * self-energy of src/gf.f90:124-148 over nocc occupied orbitals, until
 * |E - E_old| < tolE; E gets the pole, niter (may be NULL) the iterations.
 * HFGPU_ERR_NOT_CONVERGED after nscf iterations (the reference stops there).
 * FP64, from the packed MO integrals. */
int hfgpu_find_pole_diag(int n, const double *moint2, const double *lam, int nocc, int i, int nscf, double tolE,
                         double *E, int *niter);

/* FP64-accurate C = A B on the tcgen05 tensor cores (the kernel behind the
 * mixed-precision transform): A row-major M x K, Bt = B^T row-major N x K
 * (B column-major), C row-major M x N; 1 <= K <= 512.  Rows of A and columns
 * of B are split exactly into six 7-bit bf16 digits with a power-of-two scale;
 * the result agrees with an FP64 GEMM to about 2^-42 K max|A_r.| max|B_.c|. */
int hfgpu_dgemm_sliced(int64_t M, int N, int K, const double *A, const double *Bt, double *C);

/* MBPT2 energy from the packed AO integrals and the orbitals: the
 * transform_int2 + mbpt2 sequence of the reference's tests
 * (src/mbpt.f90:11-79, :154-159) without the packed MO array; only (ia|jb) is
 * formed.  precision: HFGPU_MP2_FP64 (cuBLAS DGEMM) or HFGPU_MP2_SPLIT_BF16
 * (tensor cores, exact 7-bit bf16 slicing). */
int hfgpu_mp2_energy(int n, const double *int2, const double *C, const double *lam, int nocc,
                     int precision, double *E2);

/* ---- Whole pipeline: rhf_gauss (src/drivers.f90:12-51) + MBPT2 ------------ */

enum { HFGPU_MP2_NONE = 0, HFGPU_MP2_FP64 = 1, HFGPU_MP2_SPLIT_BF16 = 2 };
enum { HFGPU_SCF_MIXING = 0, HFGPU_SCF_DIIS = 1 };

typedef struct {
    int nscf;            /* iteration cap (reference tests: 40) */
    double mix_alpha;    /* linear mixing factor (reference: 1.0, CO: 0.8) */
    double tolE;         /* energy-window tolerance (reference tests: 1e-10) */
    double tolP;         /* density-change tolerance (reference tests: 1e-8) */
    int scf_accel;       /* HFGPU_SCF_MIXING (reference algorithm) or HFGPU_SCF_DIIS */
    int diis_size;       /* DIIS history length */
    double schwarz;      /* quartet cut on sqrt((ab|ab)(cd|cd)); 0 = none (reference) */
    int mp2;             /* HFGPU_MP2_* */
    int mp2_nocc;        /* occupied orbitals passed to MBPT2; <= 0: sum(Z)/2 */
    int purify;          /* 1: density by SP2 purification (GEMMs only) in each iteration and one
                            final dsygvd for the orbitals; 0: dsygvd every iteration (reference) */
    int batch_streams;   /* hfgpu_rhf_batch: molecules in flight at once, each on its own
                            streams; <= 0: 8 */
    int incremental;     /* 1: Fock builds from density differences, each quartet's bounded
                            contribution screened at 1e-10 (or the Schwarz threshold if larger),
                            a full build every 8 iterations and near convergence; 0: full
                            builds (reference) */
    int autotune;        /* 1: time the candidate quartet-tile shapes of the ERI and Fock
                            kernels the first time a (class, size) is met and keep the
                            fastest (process-wide table); 0: built-in rules, unless the
                            environment sets HFGPU_AUTOTUNE=1 */
    int guess;           /* starting density: 0 = P = 0 (the reference's doscf), 1 = superposition
                            of free-atom densities (closer start, fewer iterations) */
    int eigensolver;     /* 0: own generalized eigensolver (as hfgpu_eigh) for 3 <= n <= 1024,
                            else cuSOLVER dsygvd; 1: cuSOLVER dsygvd always */
    int batch_mode;      /* hfgpu_rhf_batch: 0 = waves of molecules share one ERI launch and,
                            every SCF iteration, one Fock-build launch per quartet class (a
                            replayed CUDA graph), batch_streams molecules per wave at most
                            (<= 0: 32, fewer if their integrals would not fit); 1 = each molecule
                            runs the whole pipeline on its own streams, batch_streams at once */
    int reserved[1];
} hfgpu_options;

typedef struct {
    double Etot, E0, Enuc, Ekin, E2;
    double dP;               /* density change of the last iteration */
    int niter, nbf, nocc, nshell;
    int64_t n_quartets;      /* contracted shell quartets evaluated */
    int64_t n_bf_quartets;   /* unique contracted basis-function quartets evaluated */
    int64_t n_prim_quartets; /* primitive shell quartets evaluated */
    double eri_flops;        /* McMurchie-Davidson reference flop count of those */
    double ms_eri;           /* ERI class kernels (to the last of them; the SCF's set-up runs beside them) */
    double ms_scf, ms_mp2;   /* SCF set-up and loop beyond ms_eri; AO->MO transform + MBPT2 */
    double ms_total;         /* the whole call */
    double ms_setup;         /* basis, one-electron integrals, pairs, Schwarz bounds */
    double ms_fock;          /* Fock two-electron kernels summed over the SCF iterations */
    double ms_tcgemm;        /* tensor-core sliced GEMM kernels (mixed MBPT2) */
    double tc_flops;         /* bf16 tensor flops those kernels performed (2 M N K per product) */
    double ms_grad;          /* analytic gradient (hfgpu_rhf_gradient) */
    double ms_fock_full;     /* the part of ms_fock spent in full (not incremental) Fock builds */
    double n_fock_full;      /* number of those full builds */
    double block_elems;      /* component quartets a full Fock build digests (12 flops each) */
    double ms_tc_step1;      /* the tensor-core GEMMs over the packed integrals (transform step 1) */
    double n_tc_step1;       /* their launches */
    double ms_grad_eri;      /* the two-electron part of ms_grad (the ERI gradient class kernels) */
} hfgpu_result;

void hfgpu_default_options(hfgpu_options *opt);

/* natoms nuclei with charges atno at xyz (3 x natoms, bohr, column-major like
 * the reference's xyz(3, :)); 6-31G** Cartesian basis as hfsolver builds it
 * (src/basis.f90:143-569).  C (nbf x nbf) and lam (nbf) may be NULL; when
 * given they must hold nbf*nbf and nbf doubles (nbf from hfgpu_basis_size). */
int hfgpu_rhf(int natoms, const int *atno, const double *xyz, const hfgpu_options *opt,
              hfgpu_result *res, double *C, double *lam);

/* Analytic RHF nuclear gradient dE_tot/dR (Ha/bohr) at the converged SCF of
 * hfgpu_rhf with the same arguments: grad holds 3 x natoms doubles (x, y, z
 * of each atom, the layout of xyz).  The reference has no gradient; this is
 * the force callback its md.f90 integrators take (src/md.f90:13-20, forces =
 * -grad).  One- and two-electron derivative integrals are contracted with the
 * density and energy-weighted density on the GPU and never stored; the
 * two-electron part runs over the quartets that survive opt->schwarz.
 * res gets the energies (and E2 if opt->mp2 asks for it).  Returns
 * HFGPU_ERR_NOT_CONVERGED, with grad untouched, if the SCF did not converge. */
int hfgpu_rhf_gradient(int natoms, const int *atno, const double *xyz, const hfgpu_options *opt,
                       hfgpu_result *res, double *grad);

/* hfgpu_rhf for nmol molecules in one call: molecule m has natoms[m] atoms, its
 * charges and coordinates follow those of molecule m-1 in atno and xyz; res[m]
 * gets its results (res[m].niter = -status if it failed).  The molecules run in
 * waves (opt->batch_mode 0, by decreasing size): the integrals of a wave are one
 * launch per quartet class, and every SCF iteration one batched Fock build
 * serves every molecule of the wave still iterating, while each molecule's own
 * SCF steps (DIIS, density, convergence test) run on its own streams.  With
 * batch_mode 1, opt->batch_streams molecules run at once, each on its own CUDA
 * streams and library handles.  Returns the first failure's status (in
 * molecule order), or HFGPU_OK. */
int hfgpu_rhf_batch(int nmol, const int *natoms, const int *atno, const double *xyz,
                    const hfgpu_options *opt, hfgpu_result *res);

/* The autotuner's table as text, one line per tuned (kernel, quartet class,
 * size bucket): "<eri|digest> <bra pair type> <ket pair type> <log2 quartets>
 * <choice>" (choice: primitive quartets per lane for eri, lanes per quartet for
 * digest).  Writes at most len bytes including the terminating NUL and returns
 * the length of the whole text. */
int64_t hfgpu_autotune_table(char *buf, int64_t len);
/* forget every tuned shape */
void hfgpu_autotune_clear(void);

/* number of basis functions hfgpu_rhf will use for these atoms (0 on error) */
int hfgpu_basis_size(int natoms, const int *atno);

/* ---- Diagnostics: device routines of the kernels, one at a time ------------ */

/* The Boys function F_0(T) .. F_maxm(T) (0 <= maxm <= 12) for nt values T[t] >= 0,
 * evaluated by the device routine the ERI kernels use: F[t (maxm+1) + m] =
 * F_m(T[t]).  The same quantity as the reference's Fm
 * (src/special_functions.f90:189-248, called through src/cints.c:28-33);
 * host arrays.  HFGPU_ERR_INVALID for T < 0 or non-finite, as the reference
 * stops there (src/special_functions.f90:218-221). */
int hfgpu_boys(int maxm, int64_t nt, const double *T, double *F);

/* The bounded grid barrier of the cooperative SP2 and tridiagonalisation
 * kernels, with a caller-set time limit: launched_blocks blocks (at most one
 * per SM, so all are resident) arrive at a barrier that waits for
 * expected_blocks.  HFGPU_OK when the barrier completed; with fewer blocks
 * launched than expected the wait runs out after limit_ms (0 < limit_ms <=
 * 2000), every block returns with the error flag set and the call returns
 * HFGPU_ERR_CUDA, the device staying usable.  elapsed_ms (may be NULL) gets
 * the kernel's duration.  No counterpart in the reference, which has no device
 * code; it tests the failure path that replaces a hang. */
int hfgpu_grid_barrier_check(int launched_blocks, int expected_blocks, double limit_ms, double *elapsed_ms);

#ifdef __cplusplus
}
#endif

#endif /* HFGPU_H */
