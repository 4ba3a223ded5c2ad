// Generalized symmetric-definite eigensolver F C = S C diag(lam), the SCF's
// eigh (reference: deigh_generalized, src/linalg.f90:241-275, LAPACK dsygvd with
// the lower triangles; called by src/scf.f90:118-119).
//
// cuSOLVER's dsygvd spends ~8 ms on a 200 x 200 problem, almost all of it in
// launch and synchronisation latency.  Here:
//   1. F' = X^T F X with X = L^-T (S = L L^T), two DGEMMs;
//   2. Householder tridiagonalisation Q^T F' Q = T in ONE cooperative kernel:
//      one warp per block, block b keeping rows b, b + G, b + 2G, ... of the
//      trailing matrix in shared memory, one grid barrier per column (below);
//   3. T = Z diag(lam) Z^T on the host (tridiag.cpp, O(n^2));
//   4. C = X Q Z with Q = H_0 ... H_{n-3} = I - V Tw V^T in compact WY form,
//      Tw^-1 = diag(1/tau) + strict upper part of V^T V; M = X V Tw is formed
//      while the host works, so C = X Z - M (V^T Z) is three GEMMs after it.
// Step 2, column k (H_k = I - tau v v^T acting on rows k+1 .. n-1, v[k+1] = 1,
// the convention of LAPACK's dsytd2):
//   * every block holds row k of the current matrix (xs) and forms v, tau with
//     identical arithmetic, so no exchange is needed for them;
//   * the owners compute their entries of p = tau A22 v and publish them;
//   * grid barrier;
//   * every block reads p, forms w = p - (tau/2)(p.v) v and applies
//     A22 -= v w^T + w v^T to its own rows and to its private copy of row k+1,
//     which the owner of row k+1 published one column earlier; the owner of
//     row k+2 publishes it for the next column.
// p and the published row alternate between two buffers by column parity: a
// block can only reuse a buffer after the barrier of the next column, which
// every block reaches after it has finished reading that buffer.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "eigh.h"
#include "gridsync.cuh"

namespace hfgpu {

namespace {

__device__ __forceinline__ double warp_sum(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// grid barrier for one-warp blocks (gridsync.cuh)
__device__ bool trd_barrier(TrdSync* s, unsigned nblocks, unsigned epoch)
{
    __syncwarp();
    int ok = 1;
    if (threadIdx.x == 0) ok = grid_arrive_wait(&s->count, &s->err, nblocks, epoch);
    ok = __shfl_sync(0xffffffffu, ok, 0);
    return ok != 0;
}

// A: n x n symmetric (both triangles), read only.  Outputs: V (n x (n-2)
// reflectors, zero above their leading 1, an all-zero column where tau = 0),
// tau (n-2), d (n), e (n-1).  pbuf, pub: 2 n doubles each.
__global__ void __launch_bounds__(32) trd_kernel(int n, const double* __restrict__ A, double* V, double* tau,
                                                 double* d, double* e, double* pbuf, double* pub, TrdSync* sync)
{
    extern __shared__ double sm[];
    const int G = gridDim.x, b = blockIdx.x, lane = threadIdx.x;
    const int rpb = (n + G - 1) / G;
    const int nown = b < n ? (n - b + G - 1) / G : 0;
    double* rows = sm;                    // rpb x n: rows b + r G
    double* vs = rows + (size_t)rpb * n;  // reflector, indexed by column
    double* ws = vs + n;                  // p, then w
    double* xs = ws + n;                  // row k of the current matrix
    double* rs = xs + n;                  // the published row k+1, fetched with p
    for (int r = 0; r < nown; ++r) {
        const double* src = A + (size_t)(b + r * G) * n;  // column = row (symmetric)
        for (int j = lane; j < n; j += 32) rows[(size_t)r * n + j] = src[j];
    }
    for (int j = lane; j < n; j += 32) xs[j] = A[j];
    __syncwarp();

    for (int k = 0; k + 2 < n; ++k) {
        const int base = k + 1;
        // reflector of x = xs[base .. n), identical in every block
        double s2 = 0.0;
        for (int j = base + 1 + lane; j < n; j += 32) s2 = fma(xs[j], xs[j], s2);
        s2 = warp_sum(s2);
        const double alpha = xs[base];
        double t = 0.0, beta = alpha, scale = 0.0;
        if (s2 != 0.0) {
            beta = -copysign(sqrt(fma(alpha, alpha, s2)), alpha);
            t = (beta - alpha) / beta;
            scale = 1.0 / (alpha - beta);
        }
        for (int j = lane; j < n; j += 32) vs[j] = j < base ? 0.0 : (j == base ? 1.0 : xs[j] * scale);
        if (b == 0) {
            for (int j = lane; j < n; j += 32) V[(size_t)k * n + j] = t == 0.0 ? 0.0 : vs[j];
            if (lane == 0) {
                tau[k] = t;
                d[k] = xs[k];
                e[k] = beta;
            }
        }
        __syncwarp();
        // p_i = tau (A22 v)_i for the rows this block owns
        double* pk = pbuf + (size_t)(k & 1) * n;
        for (int r = 0; r < nown; ++r) {
            const int i = b + r * G;
            if (i < base) continue;
            const double* row = rows + (size_t)r * n;
            double acc = 0.0;
            for (int j = base + lane; j < n; j += 32) acc = fma(row[j], vs[j], acc);
            acc = warp_sum(acc);
            if (lane == 0) pk[i] = t * acc;
        }
        if (!trd_barrier(sync, G, (unsigned)k + 1)) return;
        // w = p - (tau/2)(p.v) v; the published row k+1 (as it was before this
        // column) is fetched in the same pass, so its L2 latency overlaps p's
        const double* prow = k == 0 ? A + n : pub + (size_t)(k & 1) * n;
        double pv = 0.0;
        for (int j = base + lane; j < n; j += 32) {
            const double p = __ldcg(pk + j);
            rs[j] = __ldcg(prow + j);
            ws[j] = p;
            pv = fma(p, vs[j], pv);
        }
        pv = warp_sum(pv);
        const double K = -0.5 * t * pv;
        for (int j = base + lane; j < n; j += 32) ws[j] = fma(K, vs[j], ws[j]);
        __syncwarp();
        // own rows: A22 -= v w^T + w v^T
        for (int r = 0; r < nown; ++r) {
            const int i = b + r * G;
            if (i < base) continue;
            double* row = rows + (size_t)r * n;
            const double vi = vs[i], wi = ws[i];
            for (int j = base + lane; j < n; j += 32) row[j] -= fma(vi, ws[j], wi * vs[j]);
        }
        // row k+1 of the updated matrix (v[base] = 1)
        const double w0 = ws[base];
        for (int j = base + lane; j < n; j += 32) xs[j] = rs[j] - fma(w0, vs[j], ws[j]);
        // the owner of row k+2 publishes it for the next column
        const int nxt = base + 1;
        if (nxt < n && nxt % G == b) {
            const double* row = rows + (size_t)((nxt - b) / G) * n;
            double* dst = pub + (size_t)((k + 1) & 1) * n;
            for (int j = nxt + lane; j < n; j += 32) dst[j] = row[j];
        }
        __syncwarp();
    }
    // the trailing 2 x 2 block: row n-2 is xs, d[n-1] from the owner of row n-1
    if (b == 0 && lane == 0) {
        d[n - 2] = xs[n - 2];
        e[n - 2] = xs[n - 1];
    }
    if ((n - 1) % G == b && lane == 0) d[n - 1] = rows[(size_t)((n - 1 - b) / G) * n + n - 1];
}

// Tw^-1 from G = V^T V (upper triangle): diagonal 1/tau (1 where tau = 0 and the
// reflector column is zero), strict upper part as is
__global__ void wy_tinv_kernel(int m, const double* __restrict__ tau, double* Tinv)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) Tinv[(size_t)k * m + k] = tau[k] != 0.0 ? 1.0 / tau[k] : 1.0;
}

// Tw = (Tw^-1)^-1 for the upper triangular Tw^-1 (m x m, column-major; its
// strict lower part is not read).  Block j forms column j by column-oriented
// back substitution of U x = e_j; the strict lower part of Tw is set to zero.
__global__ void wy_tw_kernel(int m, const double* __restrict__ Tinv, double* Tw)
{
    extern __shared__ double x[];
    const int j = blockIdx.x;
    for (int i = threadIdx.x; i < m; i += blockDim.x) x[i] = i == j ? 1.0 : 0.0;
    __syncthreads();
    for (int i = j; i >= 0; --i) {
        const double xi = x[i] / Tinv[(size_t)i * m + i];
        __syncthreads();  // every thread has read x[i]
        if (threadIdx.x == 0) x[i] = xi;
        const double* col = Tinv + (size_t)i * m;
        for (int k = threadIdx.x; k < i; k += blockDim.x) x[k] = fma(-xi, col[k], x[k]);
        __syncthreads();
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) Tw[(size_t)j * m + i] = i <= j ? x[i] : 0.0;
}

// symmetric copy of the lower triangle (the drop-in eigh reads only that)
__global__ void sym_from_lower_kernel(int n, const double* __restrict__ A, double* B)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    const int i = (int)(idx % n), j = (int)(idx / n);
    B[idx] = i >= j ? A[idx] : A[(size_t)i * n + j];
}

__global__ void identity_fill_kernel(int n, double* X)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    X[idx] = (idx % n) == (idx / n) ? 1.0 : 0.0;
}

constexpr int TRD_MAX_N = 1024;

int trd_blocks(const Context& ctx, int n) { return std::max(1, std::min(ctx.num_sms, n / 2)); }

size_t trd_smem(int n, int G) { return ((size_t)(n + G - 1) / G + 4) * n * sizeof(double); }

}  // namespace

void cholesky_orthogonalizer(Context& ctx, int n, const double* dS, double* dX)
{
    cudaStream_t st = ctx.stream;
    const int64_t nn = (int64_t)n * n;
    DBuf<double> L(nn, st);
    DBuf<int> info(1, st);
    HF_CUDA(cudaMemcpyAsync(L.p, dS, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    int lwork = 0;
    HF_CUSOLVER(cusolverDnDpotrf_bufferSize(ctx.solver, CUBLAS_FILL_MODE_LOWER, n, L.p, n, &lwork));
    DBuf<double> work(std::max(lwork, 1), st);
    HF_CUSOLVER(cusolverDnDpotrf(ctx.solver, CUBLAS_FILL_MODE_LOWER, n, L.p, n, work.p, lwork, info.p));
    int hinfo = 0;
    info.download(&hinfo, 1);
    HF_CUDA(cudaStreamSynchronize(st));
    HF_CHECK(hinfo == 0, HFGPU_ERR_LINALG, "S is not positive definite");
    identity_fill_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(n, dX);
    count_launch();
    const double one = 1.0;
    // L^T X = I
    HF_CUBLAS(cublasDtrsm(ctx.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n, n,
                          &one, L.p, n, dX, n));
}

bool Eigh::supported(Context& ctx, int n)
{
    if (n < 3 || n > TRD_MAX_N) return false;
    static std::once_flag once;
    static bool attr_ok = false;
    std::call_once(once, [] {
        attr_ok = cudaFuncSetAttribute(trd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
                  cudaSuccess;
    });
    const int G = trd_blocks(ctx, n);
    const size_t smem = trd_smem(n, G);
    if (!attr_ok || smem > 200 * 1024) return false;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trd_kernel, 32, smem) != cudaSuccess) return false;
    return (int64_t)per_sm * ctx.num_sms >= G;
}

void Eigh::setup(Context& ctx, int n_)
{
    n = n_;
    cudaStream_t st = ctx.stream;
    const int64_t nn = (int64_t)n * n;
    const int m = n - 2;
    Fp.alloc(nn, st);
    T1.alloc(nn, st);
    V.alloc((size_t)n * m, st);
    tau.alloc(m, st);
    de.alloc(2 * n, st);
    xch.alloc(4 * n, st);
    Tinv.alloc((size_t)m * m, st);
    Tw.alloc((size_t)m * m, st);
    XV.alloc((size_t)n * m, st);
    M.alloc((size_t)n * m, st);
    W.alloc((size_t)m * n, st);
    sync.alloc(1, st);
    HF_CUDA(cudaMallocHost((void**)&hbuf, sizeof(double) * (3 * n + nn) + sizeof(TrdSync)));
    HF_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
}

Eigh::~Eigh()
{
    if (hbuf) cudaFreeHost(hbuf);
    if (ready) cudaEventDestroy(ready);
}

void Eigh::solve(Context& ctx, const double* X, const double* F, double* C, double* lam, int ncol)
{
    cudaStream_t st = ctx.stream;
    const int64_t nn = (int64_t)n * n;
    const int m = n - 2;
    if (ncol <= 0 || ncol > n) ncol = n;
    const double one = 1.0, zero = 0.0, mone = -1.0;
    // F' = X^T F X
    gemm(ctx, true, false, n, n, n, 1.0, X, n, F, n, 0.0, T1.p, n);
    gemm(ctx, false, false, n, n, n, 1.0, T1.p, n, X, n, 0.0, Fp.p, n);
    ctx.trace_mark("eigh X^T F X");
    // tridiagonalisation
    {
        HF_CUDA(cudaMemsetAsync(sync.p, 0, sizeof(TrdSync), st));
        const int G = trd_blocks(ctx, n);
        const size_t smem = trd_smem(n, G);
        int n_ = n;
        const double* a = Fp.p;
        double *v = V.p, *t = tau.p, *dd = de.p, *ee = de.p + n, *pb = xch.p, *pu = xch.p + 2 * n;
        TrdSync* sy = sync.p;
        void* args[] = {&n_, &a, &v, &t, &dd, &ee, &pb, &pu, &sy};
        HF_CUDA(cudaLaunchCooperativeKernel((const void*)trd_kernel, dim3(G), dim3(32), args, smem, st));
        count_launch();
    }
    double* hd = hbuf;
    double* he = hbuf + n;
    double* hlam = hbuf + 2 * n;
    double* hZ = hbuf + 3 * n;
    TrdSync* hs = reinterpret_cast<TrdSync*>(hbuf + 3 * n + nn);
    HF_CUDA(cudaMemcpyAsync(hd, de.p, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
    HF_CUDA(cudaMemcpyAsync(hs, sync.p, sizeof(TrdSync), cudaMemcpyDeviceToHost, st));
    HF_CUDA(cudaEventRecord(ready, st));
    // while the host solves T: M = X V Tw, so that C = X Q Z = X Z - M (V^T Z)
    HF_CUBLAS(cublasDsyrk(ctx.blas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, m, n, &one, V.p, n, &zero, Tinv.p, m));
    wy_tinv_kernel<<<(m + 127) / 128, 128, 0, st>>>(m, tau.p, Tinv.p);
    count_launch();
    wy_tw_kernel<<<m, 128, (size_t)m * sizeof(double), st>>>(m, Tinv.p, Tw.p);
    count_launch();
    gemm(ctx, false, false, n, m, n, 1.0, X, n, V.p, n, 0.0, XV.p, n);
    gemm(ctx, false, false, n, m, m, 1.0, XV.p, n, Tw.p, m, 0.0, M.p, n);
    HF_CUDA(cudaEventSynchronize(ready));
    ctx.trace_mark("eigh tridiag");
    HF_CHECK(hs->err == 0, HFGPU_ERR_CUDA, "eigh: tridiagonalisation grid barrier timed out");
    tridiag_eigen(n, hd, he, hlam, hZ, ncol);
    ctx.trace_mark("eigh host");
    // Z (n x ncol) to the device, lam
    HF_CUDA(cudaMemcpyAsync(T1.p, hZ, sizeof(double) * n * ncol, cudaMemcpyHostToDevice, st));
    HF_CUDA(cudaMemcpyAsync(lam, hlam, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    // W = V^T Z; C = X Z - M W
    gemm(ctx, true, false, m, ncol, n, 1.0, V.p, n, T1.p, n, 0.0, W.p, m);
    gemm(ctx, false, false, n, ncol, n, 1.0, X, n, T1.p, n, 0.0, C, n);
    gemm(ctx, false, false, n, ncol, m, -1.0, M.p, n, W.p, m, 1.0, C, n);
    ctx.trace_mark("eigh back");
    // the next solve writes the host buffers only after its own event, which
    // follows these uploads on the stream
}

void eigh_generalized(Context& ctx, int n, const double* dA, const double* dB, double* dC, double* dLam, int solver)
{
    cudaStream_t st = ctx.stream;
    const int64_t nn = (int64_t)n * n;
    DBuf<double> As(nn, st);
    sym_from_lower_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(n, dA, As.p);
    count_launch();
    if (solver == 0 && Eigh::supported(ctx, n)) {
        DBuf<double> X(nn, st);
        cholesky_orthogonalizer(ctx, n, dB, X.p);
        Eigh e;
        e.setup(ctx, n);
        e.solve(ctx, X.p, As.p, dC, dLam);
        HF_CUDA(cudaStreamSynchronize(st));
        return;
    }
    DBuf<double> Bw(nn, st);
    DBuf<int> info(1, st);
    HF_CUDA(cudaMemcpyAsync(dC, As.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    HF_CUDA(cudaMemcpyAsync(Bw.p, dB, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    int lwork = 0;
    HF_CUSOLVER(cusolverDnDsygvd_bufferSize(ctx.solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                            CUBLAS_FILL_MODE_LOWER, n, dC, n, Bw.p, n, dLam, &lwork));
    DBuf<double> work(std::max(lwork, 1), st);
    HF_CUSOLVER(cusolverDnDsygvd(ctx.solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                 dC, n, Bw.p, n, dLam, work.p, lwork, info.p));
    int hinfo = 0;
    info.download(&hinfo, 1);
    HF_CUDA(cudaStreamSynchronize(st));
    HF_CHECK(hinfo == 0, HFGPU_ERR_LINALG, "eigh: dsygvd returned info = " + std::to_string(hinfo));
}

}  // namespace hfgpu
