// Internal declarations shared by the libhfgpu translation units.
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/hfgpu.h"

namespace hfgpu {

// ---------------------------------------------------------------- errors
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& m);

#define HF_CUDA(x)                                                                             \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess)                                                                 \
            throw ::hfgpu::Error(e_ == cudaErrorMemoryAllocation ? HFGPU_ERR_NOMEM            \
                                                                  : HFGPU_ERR_CUDA,           \
                                 std::string(#x) + ": " + cudaGetErrorString(e_));             \
    } while (0)
#define HF_CUBLAS(x)                                                                           \
    do {                                                                                       \
        cublasStatus_t s_ = (x);                                                               \
        if (s_ != CUBLAS_STATUS_SUCCESS)                                                       \
            throw ::hfgpu::Error(HFGPU_ERR_CUDA, std::string(#x) + ": cublas status " +       \
                                                     std::to_string((int)s_));                 \
    } while (0)
#define HF_CUSOLVER(x)                                                                         \
    do {                                                                                       \
        cusolverStatus_t s_ = (x);                                                             \
        if (s_ != CUSOLVER_STATUS_SUCCESS)                                                     \
            throw ::hfgpu::Error(HFGPU_ERR_CUDA, std::string(#x) + ": cusolver status " +     \
                                                     std::to_string((int)s_));                 \
    } while (0)
#define HF_CHECK(cond, code, msg)                                                              \
    do {                                                                                       \
        if (!(cond)) throw ::hfgpu::Error(code, msg);                                          \
    } while (0)

// ---------------------------------------------------------------- device buffers
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    DBuf() = default;
    DBuf(size_t count, cudaStream_t s) { alloc(count, s); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), st(o.st) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept
    {
        release();
        p = o.p; n = o.n; st = o.st;
        o.p = nullptr; o.n = 0;
        return *this;
    }
    void alloc(size_t count, cudaStream_t s)
    {
        release();
        st = s;
        n = count;
        if (count) HF_CUDA(cudaMallocAsync((void**)&p, count * sizeof(T), s));
    }
    void zero() { if (n) HF_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), st)); }
    void upload(const T* h, size_t count)
    {
        if (count) HF_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
    }
    void upload(const std::vector<T>& v)
    {
        if (v.size() > n) alloc(v.size(), st);
        upload(v.data(), v.size());
    }
    void download(T* h, size_t count) const
    {
        if (count) HF_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, st));
    }
    void release()
    {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        n = 0;
    }
    ~DBuf() { release(); }
};

template <class T>
DBuf<T> to_device(const std::vector<T>& v, cudaStream_t s)
{
    DBuf<T> b(v.size(), s);
    b.upload(v.data(), v.size());
    return b;
}

// ---------------------------------------------------------------- context
// One per CUDA device, created on first use: stream, library handles and the
// Boys-function grid.
struct Context {
    int device = -1;
    cudaStream_t stream = nullptr;      // the stream every call runs on
    cudaStream_t own_stream = nullptr;  // the library's own stream
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
    double* boys = nullptr;  // device copy of the Boys grid
    int num_sms = 0;
    // side streams for independent launches (quartet classes), joined back to
    // `stream` by events
    static constexpr int NAUX = 8;
    cudaStream_t aux[NAUX] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[NAUX] = {};
    void fork();  // aux streams wait for the work queued so far on `stream`
    void join();  // `stream` waits for the work queued on the aux streams
    // event pairs around Fock builds, summed into stat_fock_ms by settle_timers()
    // once the stream is synchronised anyway (no host wait per build)
    struct FockTimer {
        cudaEvent_t a, b;
        bool full;  // a full build (not a screened density difference)
    };
    std::vector<FockTimer> fock_events;
    void settle_timers();
    double stat_fock_full_ms = 0, stat_fock_full_n = 0;
    // kernel-time counters, reset by the pipeline entry points
    double stat_fock_ms = 0, stat_tc_ms = 0, stat_tc_flops = 0;
    // the gather-fed GEMM over the packed integrals (transform step 1) alone
    double stat_tc_step1_ms = 0, stat_tc_step1_n = 0;
    bool tune = false;  // time candidate kernel shapes on first use (autotune.cpp)
    // phase trace (HFGPU_TRACE=1 in the environment): an event on `stream` and a
    // host clock reading at each named point of a pipeline call; trace_report()
    // prints, per name, the device and host time since the previous point
    struct TraceMark {
        const char* name;
        cudaEvent_t ev;
        double host_ms;
    };
    bool trace_on = false;
    std::vector<TraceMark> trace;
    void trace_begin();
    void trace_mark(const char* name);
    void trace_report();
    // held by every public call for its whole duration: calls from several host
    // threads on one context run one after another (handles and stream are shared)
    std::recursive_mutex call_mutex;
};
// C = alpha op(A) op(B) + beta C in FP64, column-major: the own small-matrix
// kernel for m, n, k <= 512 (gemm_small.cu), cuBLAS beyond
void gemm(Context& ctx, bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda,
          const double* B, int ldb, double beta, double* C, int ldc);
// algorithmic FP64 flops of one primitive shell quartet (la lb | lc ld): the fixed
// McMurchie-Davidson count of the ERI roofline (eri.cu)
double md_flops(int la, int lb, int lc, int ld);
Context& context();  // for the current device
Context* context_acquire();        // a separate context on the current device (pooled)
void context_release(Context* c);  // back to the pool
void count_launch(int n = 1);  // bookkeeping for hfgpu_kernel_launches

// ---------------------------------------------------------------- basis
// A shell: all Cartesian components of one angular momentum on one centre with
// shared exponents.  comp_fn maps each component to its basis-function index,
// or -1 for a component that the caller's function list does not contain.
struct Shell {
    int L = 0, nprim = 0;
    double x = 0, y = 0, z = 0;
    int prim0 = 0;   // offset of the exponents in Basis::alpha
    int coef0 = 0;   // offset of the ncart(L) x nprim coefficient block (component-major)
    int cfn0 = 0;    // offset in Basis::comp_fn
    int atom = -1;   // index of the nucleus it sits on (-1: not built from atoms)
};

struct Basis {
    int nbf = 0;
    std::vector<Shell> shells;
    std::vector<double> alpha, coef;
    std::vector<int> comp_fn;
    int max_l() const;
};

// hfsolver's 6-31G** Cartesian basis for the given atoms (src/basis.f90:275-488)
Basis build_basis(int natoms, const int* atno, const double* xyz);
// group a reference-style function list (qc.h arguments) into shells
Basis basis_from_functions(int nbf, const int* nprim, const int* istart, const double* xc,
                           const double* yc, const double* zc, const int* lp, const int* mp,
                           const int* np, int n2, const double* coef, const double* alpha);
int basis_size(int natoms, const int* atno);

// ---------------------------------------------------------------- integrals
struct EriStats {
    int64_t n_quartets = 0, n_bf_quartets = 0, n_prim_quartets = 0;
    int64_t n_block_elems = 0;  // component quartets of the surviving shell quartets (Fock digest work)
    double flops = 0;
    double ms = 0;
};

class EriEngine;  // eri.cu

// Device-side basis + shell pairs + screened quartet segments for one molecule.
struct EriPlan;
EriPlan* eri_plan_create(Context& ctx, const Basis& b, double schwarz);
void eri_plan_destroy(EriPlan* p);
EriStats eri_plan_stats(const EriPlan* p);
// all unique (ij|kl) into the packed array d_out (device, zeroed by the caller)
void eri_compute_packed(Context& ctx, EriPlan* p, double* d_out, EriStats* st);
// the same, d_out may be null; keep_blocks also keeps the screened quartet blocks
// in HBM for eri_digest
void eri_compute(Context& ctx, EriPlan* p, double* d_out, bool keep_blocks, EriStats* st);
void eri_compute_start(Context& ctx, EriPlan* p, double* d_out, bool keep_blocks);
void eri_compute_finish(Context& ctx, EriPlan* p, EriStats* st);
// G = J - K/2 of density dP from the kept quartet blocks (n x n); screen > 0
// leaves out quartets whose Schwarz bound times the largest |dP| element they
// touch is below screen (for density differences)
void eri_digest(Context& ctx, EriPlan* p, const double* dP, double* dG, double screen = 0.0);

// one-electron integrals (onee.cu): S, T, V on the device (n x n, symmetric)
// (on: the stream to run on, ctx.stream if null; the results are ready in stream
// order there, the host does not wait)
void onee_compute(Context& ctx, const Basis& b, int natoms, const int* atno, const double* x,
                  const double* y, const double* z, double* dS, double* dT, double* dV, cudaStream_t on = nullptr);

// J/K (jk.cu): G = J - K/2 from packed integrals and density P (device)
void jk_from_packed(Context& ctx, int n, const double* d_int2, const double* dP, double* dG);
// J and K separately: J(i,j) = sum_kl (ij|kl) P(k,l), K(i,j) = sum_kl (ik|jl) P(k,l)
void jk_separate_from_packed(Context& ctx, int n, const double* d_int2, const double* dP, double* dJ, double* dK);

int64_t packed_size(int64_t n);

// superposition of atomic densities for a basis built by build_basis (guess.cpp):
// dP0 (device, nbf x nbf) gets the block-diagonal sum of cached free-atom densities
void sad_guess(Context& ctx, int natoms, const int* atno, int nbf, double* dP0);

// analytic RHF nuclear gradient (grad.cu) at converged orbitals dC, energies dL
// (device, n x n and n); grad gets 3 values per atom (Ha/bohr), host memory
void rhf_gradient(Context& ctx, EriPlan* plan, int natoms, const int* atno, const double* xyz, const double* dC,
                  const double* dL, int nocc, double* grad, double* ms_grad, double* ms_grad_eri);

// probe.cu: measured FP64 FMA rate (TFLOP/s)
double probe_fp64_tflops(Context& ctx);

// ---------------------------------------------------------------- batches of molecules
// eri.cu: several molecules' plans merged into one (segments tagged by
// molecule), so one launch per quartet class computes or digests all of them
EriPlan* eri_plan_merge(Context& ctx, const std::vector<EriPlan*>& plans);
// device tables of a batched Fock build over a merged plan: per molecule its
// density and output pointers and its screen (< 0: not in this build), set in
// the pinned host copies h_P, h_G, h_screen before each eri_digest_batch
struct BatchDigest {
    int nmol = 0;
    DBuf<int64_t> nn_prefix, dm_prefix;  // element offsets of the molecules' n x n and ns x ns blocks
    DBuf<int> mol_n, mol_ns, mol_sh0;
    DBuf<double> Gh, Dm;                 // half matrices and shell-pair maxima of all molecules
    DBuf<double*> mol_Gh, mol_G;
    DBuf<const double*> mol_Dm, mol_P;
    DBuf<double> mol_screen;
    const double** h_P = nullptr;
    double** h_G = nullptr;
    double* h_screen = nullptr;
    cudaGraphExec_t exec = nullptr;      // the build's launches, captured on first use
    int64_t graph_kernels = 0;
    cudaEvent_t copied = nullptr;        // recorded after each build's table copies
    void setup(Context& ctx, const EriPlan* P, cudaStream_t s);
    void wait_tables();                  // host tables free to be rewritten
    ~BatchDigest();
};

// one Fock build (G = J - K/2) for every molecule with h_screen >= 0, on stream s
void eri_digest_batch(Context& ctx, EriPlan* P, BatchDigest& t, cudaStream_t s);
// kernels counted so far (context.cu)
int64_t launches_counted();

// noalloc.cu: load the module that holds the allocation-free Fock build's fixed
// scratch array on device dev (the current device) and cache its device
// address; called when a device context is created, so that the array's device
// memory is taken then and not at the first allocation-free call
void noalloc_prepare(int dev);

}  // namespace hfgpu
