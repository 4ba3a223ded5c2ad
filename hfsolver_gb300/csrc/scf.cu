// Closed-shell RHF SCF loop on the GPU.
//
// Follows doscf (src/scf.f90:72-136): P = 0 start, F = H + G(P),
// E0 = sum P (H + F) / 2, generalised eigenproblem F C = S C lam solved with
// the same LAPACK routine the reference calls (dsygvd, lower triangle,
// src/linalg.f90:241-280; here cuSOLVER's device implementation),
// P = 2 C_occ C_occ^T (formP, :12-24), dP = sqrt(sum (P - Pold)^2 / 4),
// convergence from the 4th iteration when dP < tolP and the last four energies
// span less than tolE, otherwise linear mixing P = (1-alpha) Pold + alpha P.
// Optionally Pulay's DIIS (commutator error F P S - S P F) extrapolates F
// instead of mixing P.  Everything stays on the device; each iteration reads
// back two scalars (E0, dP) for the convergence test.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "internal.h"
#include "eigh.h"
#include "gridsync.cuh"
#include "scf.h"

namespace hfgpu {

__global__ void add_kernel(int64_t nn, const double* __restrict__ A, const double* __restrict__ B, double* C)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) C[i] = A[i] + B[i];
}

__global__ void sub_kernel(int64_t nn, const double* __restrict__ A, const double* __restrict__ B, double* C)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) C[i] = A[i] - B[i];
}

__global__ void mix_kernel(int64_t nn, double alpha, const double* __restrict__ Pold, double* P)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) P[i] = (1 - alpha) * Pold[i] + alpha * P[i];
}

__global__ void comm_kernel(int n, const double* __restrict__ Y, double* E)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    int i = idx % n, j = idx / n;
    E[idx] = Y[idx] - Y[j + (int64_t)i * n];
}

// Deterministic single-block reductions (n^2 <= a few 1e5 elements).
// mode 0: sum A*(B+C)/2, mode 1: sqrt(sum (A-B)^2 / 4), mode 2: sum A*B
__global__ void reduce_kernel(int mode, int64_t nn, const double* __restrict__ A, const double* __restrict__ B,
                              const double* __restrict__ C, double* out)
{
    __shared__ double sh[1024];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < nn; i += blockDim.x) {
        if (mode == 0)
            s += A[i] * (B[i] + C[i]);
        else if (mode == 1)
            s += (A[i] - B[i]) * (A[i] - B[i]);
        else
            s += A[i] * B[i];
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double r = sh[0];
        if (mode == 0) r *= 0.5;
        if (mode == 1) r = sqrt(r / 4);
        *out = r;
    }
}

static void reduce(Context& ctx, int mode, int64_t nn, const double* A, const double* B, const double* C,
                   double* dout)
{
    reduce_kernel<<<1, 1024, 0, ctx.stream>>>(mode, nn, A, B, C, dout);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

static unsigned nblk(int64_t n) { return (unsigned)((n + 255) / 256); }

// ---- density by purification (SP2, Niklasson, Phys. Rev. B 66, 155115 (2002)) ----
// Gershgorin bounds of a symmetric matrix: b[0] <= lowest, b[1] >= highest eigenvalue.
// One warp per column (the matrix is symmetric, so column sums are row sums):
// coalesced reads, shuffle sums.
__global__ void gersh_kernel(int n, const double* __restrict__ A, double* b)
{
    __shared__ double lo[32], hi[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double l = 1e300, h = -1e300;
    for (int i = warp; i < n; i += nw) {
        const double* col = A + (int64_t)i * n;
        double r = 0;
        for (int j = lane; j < n; j += 32)
            if (j != i) r += fabs(col[j]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        const double d = col[i];
        l = fmin(l, d - r);
        h = fmax(h, d + r);
    }
    if (lane == 0) {
        lo[warp] = l;
        hi[warp] = h;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w) {
            l = fmin(l, lo[w]);
            h = fmax(h, hi[w]);
        }
        b[0] = l;
        b[1] = h;
    }
}

// X2 = X X for symmetric X (n <= 1024), upper-triangle 16x16 tiles mirrored;
// the diagonal of X2 is added to trX2 (one SP2 step's tr X^2).
constexpr int SQ_T = 16;
__global__ void __launch_bounds__(SQ_T* SQ_T) sym_square_kernel(int n, const double* __restrict__ X, double* X2,
                                                                double* trX2)
{
    __shared__ double As[SQ_T][SQ_T + 1], Bs[SQ_T][SQ_T + 1];
    // blockIdx.x -> tile pair (ti <= tj), row-major over the upper triangle
    const int nt = (n + SQ_T - 1) / SQ_T;
    int b = blockIdx.x, ti = 0;
    while (b >= nt - ti) {
        b -= nt - ti;
        ++ti;
    }
    const int tj = ti + b;
    const int ty = threadIdx.x / SQ_T, tx = threadIdx.x % SQ_T;
    const int i = ti * SQ_T + ty, j = tj * SQ_T + tx;
    double acc = 0.0;
    for (int k0 = 0; k0 < n; k0 += SQ_T) {
        const int ka = k0 + tx, kb = k0 + ty;
        As[ty][tx] = (i < n && ka < n) ? X[i + (int64_t)ka * n] : 0.0;  // X[i][k]
        Bs[ty][tx] = (kb < n && j < n) ? X[kb + (int64_t)j * n] : 0.0;  // X[k][j]
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SQ_T; ++k) acc = fma(As[ty][k], Bs[k][tx], acc);
        __syncthreads();
    }
    if (i < n && j < n) {
        X2[i + (int64_t)j * n] = acc;
        if (ti != tj) X2[j + (int64_t)i * n] = acc;
        if (i == j) atomicAdd(trX2, acc);
    }
}

// The whole SP2 recursion in one cooperative launch: one block per upper-
// triangle 16x16 tile of the iterate X, grid-wide barriers between the square
// and the update, the square-or-not choice and the convergence test made by
// every block from the same traces.  A block keeps its own tile of X^2 in
// registers, so only X travels through memory (read past L1: other blocks
// wrote it).  Every barrier wait is bounded; a timeout sets err and all blocks
// leave.
struct Sp2Sync {
    unsigned count, gen;
    int err, steps;
};

// grid barrier number `epoch` of one SP2 launch (gridsync.cuh)
__device__ bool sp2_grid_barrier(Sp2Sync* s, unsigned nblocks, unsigned epoch)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) ok = grid_arrive_wait(&s->count, &s->err, nblocks, epoch);
    __syncthreads();
    return ok;
}

// Sum of v over the block into *dst (one atomic per block).
__device__ __forceinline__ void block_add(double v, double* dst)
{
    __shared__ double part[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) part[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
        if (s != 0.0) atomicAdd(dst, s);
    }
    __syncthreads();
}

// The whole SP2 recursion as one cooperative launch, one grid barrier per step.
// tr[2k] = tr X_k and tr[2k+1] = ||X_k||_F^2 = tr X_k^2 (X_k symmetric) are
// reduced while X_k is written, so every block can choose X^2 or 2X - X^2 for
// step k before it squares.  The iterate alternates between X0 and X1; a block
// squares its tt x tt upper-triangle tile from its tt rows and tt columns of X_k,
// staged whole in shared memory (stride n + 1: no bank conflicts).  The result
// ends in X0.  T = float for the coarse steps of early SCF iterations.  The tile
// edge tt (8 .. 32) and the number of k-slices ks each output's dot product is
// split into (their partial sums meet in shared memory) are chosen so that the
// FP64 work spreads evenly over the SMs and over each SM's four sub-partitions
// (sp2_shape).
template <typename T>
__global__ void __launch_bounds__(1024) sp2_persistent_kernel(int n, int nocc, int tt, int ks, T* X0, T* X1,
                                                              double* tr, int maxs, double tol_idem, double tol_n,
                                                              Sp2Sync* sync)
{
    extern __shared__ __align__(16) unsigned char sp2_smem[];
    const int ld = n + 1;
    T* Ar = (T*)sp2_smem;  // rows i0 .. i0+tt-1 of X_k, all k
    T* Bc = Ar + tt * ld;  // columns j0 .. j0+tt-1 (rows by symmetry)
    T* part = Bc + tt * ld;  // partial dot products of k-slices 1 .. ks-1
    const int nt = (n + tt - 1) / tt;
    int b = blockIdx.x, ti = 0;
    while (b >= nt - ti) {
        b -= nt - ti;
        ++ti;
    }
    const int tj = ti + b;
    const int i0 = ti * tt, j0 = tj * tt;
    // ks x tt x tt workers: output (ty, tx) of k-slice `slice` (ks slices spread the
    // tile's FP64 work over all four sub-partitions of the SM); the block is rounded
    // up to whole warps for the reductions
    const int outs = tt * tt;
    const bool worker = (int)threadIdx.x < ks * outs;
    const int slice = (int)threadIdx.x / outs, o = (int)threadIdx.x - slice * outs;
    const int ty = o / tt, tx = o % tt;
    const int i = i0 + ty, j = j0 + tx;
    const int kc = (n + ks - 1) / ks, k0 = slice * kc, k1 = min(n, k0 + kc);
    const bool own = worker && slice == 0 && i < n && j < n;
    for (int it = 0; it < maxs; ++it) {
        T* Xc = (it & 1) ? X1 : X0;
        T* Xn = (it & 1) ? X0 : X1;
        const double t0 = __ldcg(tr + 2 * it), t1 = __ldcg(tr + 2 * it + 1);
        if (fabs(t0 - t1) < tol_idem && fabs(t0 - nocc) < tol_n) {
            if ((it & 1) && own) {  // X_k is in X1: move this block's tile to X0
                X0[i + (int64_t)j * n] = __ldcg(X1 + i + (int64_t)j * n);
                if (ti != tj) X0[j + (int64_t)i * n] = __ldcg(X1 + j + (int64_t)i * n);
            }
            if (blockIdx.x == 0 && threadIdx.x == 0) sync->steps = it;
            return;
        }
        const bool square = fabs(t1 - nocc) <= fabs(2 * t0 - t1 - nocc);
        for (int e = threadIdx.x; e < tt * n; e += blockDim.x) {
            const int r = e % tt, k = e / tt;  // r fastest: tt consecutive elements of a column
            Ar[r * ld + k] = (i0 + r < n) ? __ldcg(Xc + i0 + r + (int64_t)k * n) : T(0);
            Bc[r * ld + k] = (j0 + r < n) ? __ldcg(Xc + j0 + r + (int64_t)k * n) : T(0);
        }
        __syncthreads();
        T acc = 0;
        if (worker) {
            const T* ar = Ar + ty * ld;
            const T* bc = Bc + tx * ld;
            for (int k = k0; k < k1; ++k) acc = fma(ar[k], bc[k], acc);
            if (slice > 0) part[(slice - 1) * outs + o] = acc;
        }
        if (ks > 1) {
            __syncthreads();
            if (worker && slice == 0)
                for (int q = 1; q < ks; ++q) acc += part[(q - 1) * outs + o];
        }
        double pt = 0.0, pn = 0.0;
        if (own) {
            const T x = square ? acc : T(2) * __ldcg(Xc + i + (int64_t)j * n) - acc;
            Xn[i + (int64_t)j * n] = x;
            if (ti != tj) Xn[j + (int64_t)i * n] = x;
            if (i == j) pt = (double)x;
            pn = (double)x * (double)x * (ti != tj ? 2.0 : 1.0);
        }
        block_add(pt, tr + 2 * (it + 1));  // (its __syncthreads also guard Ar/Bc reuse)
        block_add(pn, tr + 2 * (it + 1) + 1);
        if (!sp2_grid_barrier(sync, gridDim.x, (unsigned)it + 1)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sync->steps = maxs;
}

// dst = src in another precision; trn[0] += its trace, trn[1] += its squared norm
template <typename S, typename D>
__global__ void convert_trace_kernel(int n, const S* __restrict__ src, D* __restrict__ dst, double* trn)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0, q = 0.0;
    if (idx < (int64_t)n * n) {
        const D v = (D)src[idx];
        dst[idx] = v;
        if (idx % n == idx / n) t = (double)v;
        q = (double)v * (double)v;
    }
    block_add(t, trn);
    block_add(q, trn + 1);
}

// X = (emax I - F) / (emax - emin): spectrum mapped into [0, 1], occupied states
// near 1; trX[0] = tr X and trX[1] = ||X||_F^2 of this initial iterate
__global__ void sp2_init2_kernel(int n, const double* __restrict__ F, const double* __restrict__ b, double* X,
                                 double* trX)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0, q = 0.0;
    if (idx < (int64_t)n * n) {
        const int i = idx % n, j = idx / n;
        const double x = ((i == j ? b[1] : 0.0) - F[idx]) / (b[1] - b[0]);
        X[idx] = x;
        if (i == j) t = x;
        q = x * x;
    }
    block_add(t, trX);
    block_add(q, trX + 1);
}

// one SP2 step from the traces of this step (t[0] = tr X, t[1] = tr X^2);
// accumulates tr of the new iterate into tnext[0]
__global__ void sp2_step_kernel(int n, int nocc, const double* __restrict__ t, const double* __restrict__ X2,
                                double* X, double* tnext)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    const bool square = fabs(t[1] - nocc) <= fabs(2 * t[0] - t[1] - nocc);
    const double x = square ? X2[idx] : 2 * X[idx] - X2[idx];
    X[idx] = x;
    const int i = idx % n, j = idx / n;
    if (i == j) atomicAdd(tnext, x);
}

static int sp2_threads(int tt, int ks) { return (ks * tt * tt + 31) / 32 * 32; }
static size_t sp2_smem_bytes(int n, int tt, int ks, size_t elem)
{
    return (2 * (size_t)tt * (n + 1) + (size_t)(ks - 1) * tt * tt) * elem;
}
static unsigned sp2_tiles(int n, int tt)
{
    const int nt = (n + tt - 1) / tt;
    return (unsigned)(nt * (nt + 1) / 2);
}

// can all blocks of the persistent SP2 kernel with tile edge tt be resident at once?
static bool coop_ok(Context& ctx, int n, int tt, int ks)
{
    int coop = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx.device) != cudaSuccess || !coop) return false;
    // the attribute is per process: set it once, to the most a block may have,
    // so that concurrent molecules of other sizes never lower it
    // (the block's opt-in maximum less the kernels' static shared memory)
    static std::once_flag once;
    static bool attr_ok = false;
    static size_t most = 0;
    const int dev = ctx.device;
    std::call_once(once, [dev] {
        int optin = 0;
        cudaFuncAttributes fd{}, ff{};
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fd, sp2_persistent_kernel<double>) != cudaSuccess ||
            cudaFuncGetAttributes(&ff, sp2_persistent_kernel<float>) != cudaSuccess) {
            (void)cudaGetLastError();
            return;
        }
        most = (size_t)optin - std::max(fd.sharedSizeBytes, ff.sharedSizeBytes);
        attr_ok = cudaFuncSetAttribute(sp2_persistent_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)most) == cudaSuccess &&
                  cudaFuncSetAttribute(sp2_persistent_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)most) == cudaSuccess;
        if (!attr_ok) (void)cudaGetLastError();  // no pending error for the next launch check
    });
    if (!attr_ok || n > 512 || sp2_smem_bytes(n, tt, ks, sizeof(double)) > most) return false;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sp2_persistent_kernel<double>, sp2_threads(tt, ks),
                                                      sp2_smem_bytes(n, tt, ks, sizeof(double))) != cudaSuccess)
        return false;
    return (int64_t)per_sm * ctx.num_sms >= (int64_t)sp2_tiles(n, tt);
}

// tile edge tt and k-slices ks of the persistent SP2 kernel.  Per step, a warp's
// FP64 FMA keeps its sub-partition's FP64 pipe ~64 cycles busy on this GPU, so the
// busiest sub-partition of the busiest SM takes ceil(resident warps / 4) x n/ks
// such instructions; every block adds ~40 cycles of atomics at the barrier and the
// trace sums.  Take the (tt in 8 .. 32, ks in 1 .. 4, at most 1024 threads) with
// the least of both among those whose grid can be co-resident (n = 400: edge 17
// or 25, where 8 .. 16 would need more blocks per SM than shared memory allows).
// tt = 0: none fits.
struct Sp2Shape {
    int tt = 0, ks = 1;
};

static Sp2Shape sp2_shape(Context& ctx, int n)
{
    Sp2Shape best;
    int64_t best_cost = 0;
    for (int tt = 32; tt >= 8; --tt)
        for (int ks = 1; ks <= 4; ++ks) {
            if (ks * tt * tt > 1024 || !coop_ok(ctx, n, tt, ks)) continue;
            const int64_t tiles = sp2_tiles(n, tt);
            const int64_t per_sm = (tiles + ctx.num_sms - 1) / ctx.num_sms;
            const int64_t warps = sp2_threads(tt, ks) / 32;
            const int64_t cost = (per_sm * warps + 3) / 4 * ((n + ks - 1) / ks) * 64 + 40 * tiles;
            if (best.tt == 0 || cost < best_cost) {
                best.tt = tt;
                best.ks = ks;
                best_cost = cost;
            }
        }
    return best;
}

struct Purifier {
    int n = 0, nocc = 0;
    int tile = 0;  // persistent-kernel tile edge (sp2_shape); -1: per-step fallback
    int kslices = 1;
    DBuf<double> X, T1, T2, B, tr;  // orthogonaliser S^-1/2 and work
    DBuf<float> Xf;                 // FP32 iterate of the coarse steps
    DBuf<Sp2Sync> sync;
    void setup(Context& ctx, int n_, int nocc_, const double* dS)
    {
        n = n_;
        nocc = nocc_;
        const int64_t nn = (int64_t)n * n;
        cudaStream_t st = ctx.stream;
        X.alloc(nn, st);
        T1.alloc(nn, st);
        T2.alloc(nn, st);
        B.alloc(4, st);
        tr.alloc(4, st);
        // orthogonaliser X = L^-T from the Cholesky factor S = L L^T (X^T S X = I):
        // a factorisation and a triangular solve instead of an eigensolve
        cholesky_orthogonalizer(ctx, n, dS, X.p);
    }
    // One cooperative launch of the whole recursion on the iterate Xs, with
    // barrier state slot `which` (0: FP32 steps, 1: FP64 steps).
    template <typename T>
    void run_persistent(Context& ctx, T* Xs, T* Xw, double* trs, int maxs, double tol_idem, double tol_n, int tt,
                        int which)
    {
        cudaStream_t st = ctx.stream;
        HF_CUDA(cudaMemsetAsync(sync.p + which, 0, sizeof(Sp2Sync), st));
        int n_ = n, nocc_ = nocc, tt_ = tt, ks_ = kslices;
        Sp2Sync* sp = sync.p + which;
        void* args[] = {&n_, &nocc_, &tt_, &ks_, &Xs, &Xw, &trs, &maxs, &tol_idem, &tol_n, &sp};
        HF_CUDA(cudaLaunchCooperativeKernel((const void*)sp2_persistent_kernel<T>, dim3(sp2_tiles(n, tt)),
                                            dim3(sp2_threads(tt, kslices)), args,
                                            sp2_smem_bytes(n, tt, kslices, sizeof(T)), st));
        count_launch();
    }
    // The outcome of the last cooperative purification (barrier timeouts, final
    // trace) is copied to pinned host memory without waiting; check() reads it
    // after the caller's next synchronisation.
    Sp2Sync* hsync = nullptr;
    double* htr = nullptr;
    bool pending = false;
    static constexpr int MAXS = 160;
    void check()
    {
        if (!pending) return;
        pending = false;
        HF_CHECK(hsync[0].err == 0 && hsync[1].err == 0, HFGPU_ERR_CUDA,
                 "density purification: grid barrier timed out");
        const int last = std::min(std::max(hsync[1].steps, 0), MAXS);
        HF_CHECK(fabs(htr[2 * last] - nocc) < 1e-6, HFGPU_ERR_LINALG,
                 "density purification did not converge (no gap?)");
    }
    ~Purifier()
    {
        if (hsync) cudaFreeHost(hsync);
        if (htr) cudaFreeHost(htr);
    }
    // P = 2 X proj(X^T F X) X^T: the closed-shell density of F without diagonalising it.
    // coarse: run the recursion in FP32 until tr(X - X^2) < 1e-3, then finish in
    // FP64 (a few steps); the result is idempotent to FP64 precision but its
    // occupied subspace carries FP32 rounding (~1e-7), which is fine while the
    // SCF is far from convergence.
    void density(Context& ctx, const double* dF, double* dP, bool coarse = false)
    {
        const int64_t nn = (int64_t)n * n;
        cudaStream_t st = ctx.stream;
        const double one = 1.0, zero = 0.0, two = 2.0;
        gemm(ctx, true, false, n, n, n, 1.0, X.p, n, dF, n, 0.0, T1.p, n);
        gemm(ctx, false, false, n, n, n, 1.0, T1.p, n, X.p, n, 0.0, T2.p, n);
        gersh_kernel<<<1, 1024, 0, st>>>(n, T2.p, B.p);
        count_launch();
        // per-step trace slots [step][tr X, tr X^2], zeroed once
        const int CHECK = 8;
        if (tr.n < (size_t)4 * (MAXS + 1)) tr.alloc(4 * (MAXS + 1), st);
        HF_CUDA(cudaMemsetAsync(tr.p, 0, sizeof(double) * 4 * (MAXS + 1), st));
        sp2_init2_kernel<<<nblk(nn), 256, 0, st>>>(n, T2.p, B.p, T1.p, tr.p);  // T1 = iterate
        count_launch();
        ctx.trace_mark("sp2 X^T F X");
        const int nt = (n + SQ_T - 1) / SQ_T;
        const unsigned tiles = (unsigned)(nt * (nt + 1) / 2);  // of the per-step fallback
        double h[2] = {0, 1};
        bool done = false;
        if (tile == 0) {
            const Sp2Shape sh = sp2_shape(ctx, n);
            tile = sh.tt == 0 ? -1 : sh.tt;
            kslices = sh.ks;
        }
        if (tile > 0) {
            if (!sync.p) {
                sync.alloc(2, st);
                HF_CUDA(cudaMemsetAsync(sync.p, 0, 2 * sizeof(Sp2Sync), st));
                HF_CUDA(cudaMallocHost((void**)&hsync, 2 * sizeof(Sp2Sync)));
                HF_CUDA(cudaMallocHost((void**)&htr, 2 * (MAXS + 1) * sizeof(double)));
            }
            double* tr64 = tr.p;
            if (coarse) {
                if (Xf.n < (size_t)(2 * nn)) Xf.alloc(2 * nn, st);
                double* trf = tr.p + 2 * (MAXS + 1);
                convert_trace_kernel<double, float><<<nblk(nn), 256, 0, st>>>(n, T1.p, Xf.p, trf);
                count_launch();
                run_persistent<float>(ctx, Xf.p, Xf.p + nn, trf, MAXS, 1e-3, 1e-3, tile, 0);
                ctx.trace_mark("sp2 fp32");
                HF_CUDA(cudaMemsetAsync(tr64, 0, sizeof(double) * 2 * (MAXS + 1), st));
                convert_trace_kernel<float, double><<<nblk(nn), 256, 0, st>>>(n, Xf.p, T1.p, tr64);
                count_launch();
            } else {
                HF_CUDA(cudaMemsetAsync(sync.p, 0, sizeof(Sp2Sync), st));  // no FP32 phase this time
            }
            // T2 (X^T F X) is free once the first iterate is built: the second buffer
            run_persistent<double>(ctx, T1.p, T2.p, tr64, MAXS, 1e-13 * n, 1e-6, tile, 1);
            ctx.trace_mark("sp2 fp64");
            HF_CUDA(cudaMemcpyAsync(hsync, sync.p, 2 * sizeof(Sp2Sync), cudaMemcpyDeviceToHost, st));
            HF_CUDA(cudaMemcpyAsync(htr, tr64, 2 * (MAXS + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
            pending = true;
            done = true;
            h[0] = nocc;  // checked later by check()
        }
        // launch-per-step fallback: tr[2k+1] is accumulated by the square kernel
        if (!done) HF_CUDA(cudaMemsetAsync(tr.p + 1, 0, sizeof(double), st));
        for (int it = 0; it < MAXS && !done; ++it) {
            sym_square_kernel<<<tiles, SQ_T * SQ_T, 0, st>>>(n, T1.p, T2.p, tr.p + 2 * it + 1);
            count_launch();
            sp2_step_kernel<<<nblk(nn), 256, 0, st>>>(n, nocc, tr.p + 2 * it, T2.p, T1.p, tr.p + 2 * (it + 1));
            count_launch();
            if (it % CHECK == CHECK - 1) {
                // traces of step it (tr X, tr X^2) are complete once its kernels ran
                HF_CUDA(cudaMemcpyAsync(h, tr.p + 2 * it, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
                HF_CUDA(cudaStreamSynchronize(st));
                done = fabs(h[0] - h[1]) < 1e-13 * n && fabs(h[0] - nocc) < 1e-6;
            }
        }
        HF_CHECK(fabs(h[0] - nocc) < 1e-6, HFGPU_ERR_LINALG, "density purification did not converge (no gap?)");
        gemm(ctx, false, false, n, n, n, 1.0, X.p, n, T1.p, n, 0.0, T2.p, n);
        gemm(ctx, false, true, n, n, n, 2.0, T2.p, n, X.p, n, 0.0, dP, n);
    }
};

// P = 2 C_occ C_occ^T
static void form_density(Context& ctx, int n, int nocc, const double* C, double* P)
{
    const double two = 2.0, zero = 0.0;
    if (nocc == 0) {
        HF_CUDA(cudaMemsetAsync(P, 0, sizeof(double) * n * n, ctx.stream));
        return;
    }
    gemm(ctx, false, true, n, n, nocc, 2.0, C, n, C, n, 0.0, P, n);
}

// small dense solve with partial pivoting (DIIS system, size <= 21)
// The DIIS step on the device (one thread), so that the SCF iteration needs no
// host round trip for it: Bd (nd x nd) keeps <e_k, e_l>; its row and column
// `head` come from bvec (<e_k, e_head>, k < nhist).  The system
// [[B / scale, -1], [-1, 0]] c = [0 .. 0, -1] is solved by Gaussian elimination
// with partial pivoting; cvec receives the nhist coefficients, or selects the
// newest Fock matrix alone when the system is singular.
constexpr int DIIS_MAX = 20;  // the history length run_scf allows
__global__ void diis_solve_kernel(int nd, int nhist, int head, double* __restrict__ Bd,
                                  const double* __restrict__ bvec, double* __restrict__ cvec)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int k = 0; k < nhist; k++) {
        Bd[head * nd + k] = bvec[k];
        Bd[k * nd + head] = bvec[k];
    }
    const int m = nhist + 1;
    double A[(DIIS_MAX + 1) * (DIIS_MAX + 1)], b[DIIS_MAX + 1];
    double scale = 0;
    for (int a = 0; a < nhist; a++) scale = fmax(scale, fabs(Bd[a * nd + a]));
    if (scale <= 0) scale = 1;
    for (int a = 0; a < m; a++) {
        for (int c = 0; c < m; c++) A[a * m + c] = 0.0;
        b[a] = 0.0;
    }
    for (int a = 0; a < nhist; a++) {
        for (int c = 0; c < nhist; c++) A[a * m + c] = Bd[a * nd + c] / scale;
        A[a * m + nhist] = -1;
        A[nhist * m + a] = -1;
    }
    b[nhist] = -1;
    bool ok = true;
    for (int c = 0; c < m && ok; c++) {
        int piv = c;
        for (int r = c + 1; r < m; r++)
            if (fabs(A[r * m + c]) > fabs(A[piv * m + c])) piv = r;
        if (fabs(A[piv * m + c]) < 1e-300) {
            ok = false;
            break;
        }
        if (piv != c) {
            for (int k = 0; k < m; k++) {
                const double t = A[c * m + k];
                A[c * m + k] = A[piv * m + k];
                A[piv * m + k] = t;
            }
            const double t = b[c];
            b[c] = b[piv];
            b[piv] = t;
        }
        for (int r = c + 1; r < m; r++) {
            const double f = A[r * m + c] / A[c * m + c];
            for (int k = c; k < m; k++) A[r * m + k] -= f * A[c * m + k];
            b[r] -= f * b[c];
        }
    }
    if (ok)
        for (int c = m - 1; c >= 0; c--) {
            double sum = b[c];
            for (int k = c + 1; k < m; k++) sum -= A[c * m + k] * b[k];
            b[c] = sum / A[c * m + c];
        }
    for (int k = 0; k < nd; k++) cvec[k] = ok ? (k < nhist ? b[k] : 0.0) : (k == head ? 1.0 : 0.0);
}

ScfOut run_scf(Context& ctx, const ScfIn& in, double* dC, double* dP, double* dLam)
{
    cudaStream_t st = ctx.stream;
    const int n = in.n;
    const int64_t nn = (int64_t)n * n;
    HF_CHECK(in.nocc >= 0 && in.nocc <= n, HFGPU_ERR_INVALID, "nocc out of range");
    if (in.begin) in.begin(in.hook_user);
    DBuf<double> G(nn, st), F(nn, st), Fw(nn, st), Sw(nn, st), Pold(nn, st), scal(4, st);
    DBuf<int> info(1, st);
    info.zero();  // written by dsygvd; the own eigensolver reports errors by exception
    if (in.dP0)
        HF_CUDA(cudaMemcpyAsync(dP, in.dP0, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    else
        HF_CUDA(cudaMemsetAsync(dP, 0, sizeof(double) * nn, st));
    int lwork = 0;
    HF_CUSOLVER(cusolverDnDsygvd_bufferSize(ctx.solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                            CUBLAS_FILL_MODE_LOWER, n, Fw.p, n, Sw.p, n, dLam, &lwork));
    DBuf<double> work(std::max(lwork, 1), st);

    const bool diis = in.accel == HFGPU_SCF_DIIS;
    const int nd = std::max(2, std::min(in.diis_size, 20));
    DBuf<double> Fh, Eh, Y, bvec, cvec, Bd;
    if (diis) {
        Fh.alloc((size_t)nd * nn, st);
        Eh.alloc((size_t)nd * nn, st);
        Y.alloc(nn, st);
        bvec.alloc(nd, st);
        cvec.alloc(nd, st);
        Bd.alloc((size_t)nd * nd, st);
        Bd.zero();
    }
    int nhist = 0, head = 0;

    Purifier pur;
    if (in.purify) pur.setup(ctx, n, in.nocc, in.dS);
    // eigensolver: our own (eigh.cu) where it fits, with the purifier's X or one
    // made here; cuSOLVER's dsygvd otherwise
    Eigh eig;
    DBuf<double> Xown;
    const double* Xorth = nullptr;
    const bool own_eigh = in.eigensolver == 0 && Eigh::supported(ctx, n);
    if (own_eigh) {
        eig.setup(ctx, n);
        if (in.purify) {
            Xorth = pur.X.p;
        } else {
            Xown.alloc(nn, st);
            cholesky_orthogonalizer(ctx, n, in.dS, Xown.p);
            Xorth = Xown.p;
        }
    }
    // orbitals C (may alias F) and energies of F C = S C diag(lam); with the own
    // eigensolver only the lowest ncol orbitals are formed (ncol <= 0: all)
    auto eigh = [&](const double* Fm, double* Cm, int ncol) {
        if (own_eigh) {
            eig.solve(ctx, Xorth, Fm, Cm, dLam, ncol);
            return;
        }
        if (Cm != Fm) HF_CUDA(cudaMemcpyAsync(Cm, Fm, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
        HF_CUDA(cudaMemcpyAsync(Sw.p, in.dS, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
        HF_CUSOLVER(cusolverDnDsygvd(ctx.solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                     n, Cm, n, Sw.p, n, dLam, work.p, lwork, info.p));
    };

    std::vector<double> Escf;
    ScfOut out;
    // incremental Fock builds: Gacc = G(Pacc); each iteration adds G(P - Pacc)
    const bool inc = in.direct_jk && in.inc_screen > 0;
    DBuf<double> Gacc, Pacc;
    if (inc) {
        Gacc.alloc(nn, st);
        Pacc.alloc(nn, st);
    }
    // near convergence (dP < 100 tolP) every build is a full one, so the last
    // iterations converge exactly like the full-build SCF
    int since_full = 0;
    bool last_full = true, endgame = false;
    double last_dP = 1.0;
    const double* last_F = nullptr;  // the Fock matrix of the last eigensolve
    ctx.trace_mark("scf setup");
    if (in.end) in.end(in.hook_user);
    for (int it = 1; it <= in.nscf; ++it) {
        const double* Gcur = G.p;
        if (inc) {
            last_full = it == 1 || endgame || since_full >= in.inc_rebuild;
            if (last_full) {
                in.direct_jk(ctx, in.direct_ctx, dP, Gacc.p, 0.0);
                since_full = 0;
            } else {
                sub_kernel<<<nblk(nn), 256, 0, st>>>(nn, dP, Pacc.p, Pacc.p);  // Pacc <- P - Pacc
                count_launch();
                in.direct_jk(ctx, in.direct_ctx, Pacc.p, G.p, in.inc_screen);
                add_kernel<<<nblk(nn), 256, 0, st>>>(nn, Gacc.p, G.p, Gacc.p);
                count_launch();
                ++since_full;
            }
            HF_CUDA(cudaMemcpyAsync(Pacc.p, dP, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
            Gcur = Gacc.p;
        } else if (in.direct_jk) {
            in.direct_jk(ctx, in.direct_ctx, dP, G.p, 0.0);
        } else {
            jk_from_packed(ctx, n, in.d_int2, dP, G.p);
        }
        ctx.trace_mark("fock");
        add_kernel<<<nblk(nn), 256, 0, st>>>(nn, in.dH, Gcur, F.p);
        count_launch();
        reduce(ctx, 0, nn, dP, in.dH, F.p, scal.p);  // E0
        const double* Fsolve = F.p;
        // the first iteration of a P = 0 start has a commutator that vanishes
        // trivially: keep it out of the DIIS history
        if (diis && (it >= 2 || in.dP0)) {
            const double one = 1.0, zero = 0.0;
            // error = F P S - S P F = Y - Y^T with Y = F P S
            gemm(ctx, false, false, n, n, n, 1.0, F.p, n, dP, n, 0.0, G.p, n);
            gemm(ctx, false, false, n, n, n, 1.0, G.p, n, in.dS, n, 0.0, Y.p, n);
            double* ek = Eh.p + (size_t)head * nn;
            comm_kernel<<<nblk(nn), 256, 0, st>>>(n, Y.p, ek);
            count_launch();
            HF_CUDA(cudaMemcpyAsync(Fh.p + (size_t)head * nn, F.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
            nhist = std::min(nhist + 1, nd);
            // new row of B: <e_k, e_head>; the DIIS system is solved on the device
            HF_CUBLAS(cublasDgemv(ctx.blas, CUBLAS_OP_T, (int)nn, nd, &one, Eh.p, (int)nn, ek, 1, &zero, bvec.p, 1));
            diis_solve_kernel<<<1, 32, 0, st>>>(nd, nhist, head, Bd.p, bvec.p, cvec.p);
            count_launch();
            HF_CUDA(cudaGetLastError());
            ctx.trace_mark("diis error");
            if (nhist >= 2) {
                HF_CUBLAS(cublasDgemv(ctx.blas, CUBLAS_OP_N, (int)nn, nhist, &one, Fh.p, (int)nn, cvec.p, 1, &zero,
                                      Y.p, 1));
                Fsolve = Y.p;
            }
            head = (head + 1) % nd;
            ctx.trace_mark("diis extrap");
        }
        HF_CUDA(cudaMemcpyAsync(Pold.p, dP, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
        if (in.purify) {
            HF_CUDA(cudaMemcpyAsync(Fw.p, Fsolve, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
            // FP32 steps while the density is still far from converged
            pur.density(ctx, Fw.p, dP, it > 1 && !endgame && last_dP > 1e-4);
            HF_CUDA(cudaMemsetAsync(info.p, 0, sizeof(int), st));
        } else {
            // the density needs the occupied orbitals only; all are formed once converged
            eigh(Fsolve, Fw.p, in.nocc);
            form_density(ctx, n, in.nocc, Fw.p, dP);
        }
        last_F = Fsolve;
        ctx.trace_mark("density");
        reduce(ctx, 1, nn, dP, Pold.p, nullptr, scal.p + 1);  // dP
        double h[2];
        int hinfo = 0;
        scal.download(h, 2);
        info.download(&hinfo, 1);
        HF_CUDA(cudaStreamSynchronize(st));
        if (in.purify) pur.check();
        ctx.trace_mark("convergence");
        HF_CHECK(hinfo == 0, HFGPU_ERR_LINALG,
                 "eigh: dsygvd returned info = " + std::to_string(hinfo) +
                     (hinfo > n ? " (S is not positive definite)" : ""));
        const double E0 = h[0], dPv = h[1];
        last_dP = dPv;
        if (dPv < 100 * in.tolP) endgame = true;
        Escf.push_back(E0);
        out.E0 = E0;
        out.dP = dPv;
        out.niter = it;
        if (it > 3) {
            double emax = *std::max_element(Escf.end() - 4, Escf.end());
            double emin = *std::min_element(Escf.end() - 4, Escf.end());
            if (dPv < in.tolP && emax - emin < in.tolE && !last_full) {
                endgame = true;  // accept convergence only on a fully built Fock matrix
            } else if (dPv < in.tolP && emax - emin < in.tolE) {
                if (in.purify) {
                    // orbitals and orbital energies of the last Fock matrix, as the reference returns them
                    eigh(Fw.p, Fw.p, 0);
                    form_density(ctx, n, in.nocc, Fw.p, dP);
                    info.download(&hinfo, 1);
                    HF_CUDA(cudaStreamSynchronize(st));
                    HF_CHECK(hinfo == 0, HFGPU_ERR_LINALG, "eigh: dsygvd returned info = " + std::to_string(hinfo));
                } else if (own_eigh && in.nocc < n) {
                    eigh(last_F, Fw.p, 0);  // the virtual orbitals too (same occupied ones)
                }
                HF_CUDA(cudaMemcpyAsync(dC, Fw.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
                HF_CUDA(cudaStreamSynchronize(st));
                ctx.trace_mark("orbitals");
                out.converged = true;
                return out;
            }
        }
        if (!diis && in.alpha != 1.0) {
            mix_kernel<<<nblk(nn), 256, 0, st>>>(nn, in.alpha, Pold.p, dP);
            count_launch();
        }
    }
    // orbitals of the last Fock matrix
    if (in.purify) eigh(Fw.p, Fw.p, 0);
    else if (own_eigh && last_F) eigh(last_F, Fw.p, 0);
    HF_CUDA(cudaMemcpyAsync(dC, Fw.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    HF_CUDA(cudaStreamSynchronize(st));
    out.converged = false;
    return out;
}

double device_dot(Context& ctx, int64_t nn, const double* A, const double* B)
{
    DBuf<double> s(1, ctx.stream);
    reduce(ctx, 2, nn, A, B, nullptr, s.p);
    double h = 0;
    s.download(&h, 1);
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
    return h;
}

}  // namespace hfgpu
