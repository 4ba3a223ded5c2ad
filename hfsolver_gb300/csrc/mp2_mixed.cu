// Mixed-precision AO -> MO transform on the tensor cores, for MBPT2.
//
// Same (ia|jb) as ao2mo_fp64 (the quantity transform_int2, src/mbpt.f90:11-79,
// feeds to term1, src/mbpt2.f90:8-31), ordered as a half transform so that
// every contraction is one "tall A times coefficient block" GEMM in the exact
// bf16-sliced form of tcgemm.cu (FP64 inputs and outputs):
//   1. Y[p][j][la]  = sum_si (mu nu|la si) C1[si, j]     p = pair(mu >= nu)
//   2. Z[p][j][b]   = sum_la Y[p][j][la] C2[la, b]
//   3. W[q][i][mu]  = sum_nu Z[pair(mu, nu)][q] C1[nu, i]    q = (j, b)
//   4. T[q][i][a]   = sum_mu W[q][i][mu] C2[mu, a]       T[j][b][i][a] = (ia|jb)
// Steps 1-2 run over blocks of pairs and steps 3-4 over blocks of q, so each
// sliced operand stays within a fixed device-memory budget.
#include <algorithm>
#include <vector>

#include "internal.h"
#include "scf.h"
#include "tcgemm.h"

namespace hfgpu {

static const int64_t SLICE_BUDGET_ROWS = 1 << 20;  // rows per sliced operand (x K_pad x 10 bytes)

// out[c][r] = in[r][c] for a rows x cols row-major matrix (32 x 32 tiles through
// shared memory, both sides coalesced)
__global__ void transpose_kernel(const double* __restrict__ in, int64_t rows, int64_t cols, double* __restrict__ out)
{
    __shared__ double t[32][33];
    const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int64_t r = r0 + y, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[y][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int64_t c = c0 + y, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[c * rows + r] = t[threadIdx.x][y];
    }
}

void transpose_device(Context& ctx, const double* in, int64_t rows, int64_t cols, double* out)
{
    const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, ctx.stream>>>(in, rows, cols, out);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

void ao2mo_sliced(Context& ctx, int n, const double* d_int2, const double* C1, int n1, const double* C2, int n2,
                  double* T)
{
    cudaStream_t st = ctx.stream;
    HF_CHECK(n <= 512, HFGPU_ERR_UNSUPPORTED, "mixed-precision transform supports up to 512 functions");
    const int64_t npair = (int64_t)n * (n + 1) / 2;
    std::vector<int2> hp(npair);
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= i; j++) hp[(size_t)i * (i + 1) / 2 + j] = make_int2(i, j);
    DBuf<int2> pairs = to_device(hp, st);
    Sliced B1, B2, A;
    // steps 2 and 4 (N = v) read their FP64 rows straight into the gather-fed GEMM
    // (coalesced rows, no slice planes through HBM) while the virtual block spans
    // at most DENSE_GATHER_TILES output tiles of 80 columns; wider ones use slicing
    // + TMA.  Measured at 16 waters (v = 320, four tiles): gathering each row four
    // times beats slicing it once through HBM (steps 2 + 4: 131 -> 91 ms).  The gather GEMM walks whole 80-column tiles of B, so C2's slices are
    // then padded to a multiple of 80 rows.
    constexpr int DENSE_GATHER_TILES = 4;
    const bool dense_gather = n2 <= 80 * DENSE_GATHER_TILES;
    slice_dense(ctx, C1, n1, n, n, B1, SLICE_TILE_B);  // rows of B^T = columns of C1
    slice_dense(ctx, C2, n2, n, n, B2, dense_gather ? 80 : SLICE_TILE_B);
    ctx.trace_mark("mp2 slice C");
    const int64_t nq = (int64_t)n1 * n2;
    // gather-fed GEMMs for steps 1 and 3 when C1's columns fit one output tile of
    // the gather kernel (64 or 80 columns); with two column tiles the rows would be
    // gathered twice and the slicing + TMA path wins
    const bool gather = n1 <= 80;
    // row maxima of the gathered rows (exponents of their slices), by coalesced
    // passes over the packed array instead of a second gather inside the GEMM
    DBuf<unsigned> rmax;
    if (gather) {
        // reused by steps 3-4 for blocks of at most qb rows q
        const int64_t qb_rows = std::max<int64_t>(1, SLICE_BUDGET_ROWS / std::max(n, n1));
        rmax.alloc((size_t)std::max(npair, std::min(qb_rows, nq)) * n, st);
        packed_row_max(ctx, d_int2, n, rmax.p);
        ctx.trace_mark("mp2 row max");
    }
    DBuf<double> Z((size_t)npair * nq, st);
    // steps 1-2 over blocks of pairs
    const int64_t pb = std::max<int64_t>(1, SLICE_BUDGET_ROWS / n);
    const int64_t qb_rows2 = std::max<int64_t>(1, SLICE_BUDGET_ROWS / std::max(n, n1));
    DBuf<unsigned> dmax;
    if (dense_gather) dmax.alloc((size_t)std::max(std::min(pb, npair), std::min(qb_rows2, nq)) * n1, st);
    DBuf<double> Y((size_t)std::min(pb, npair) * n1 * n, st);
    for (int64_t p0 = 0; p0 < npair; p0 += pb) {
        const int64_t np = std::min(pb, npair - p0);
        // rows (p, la) -> Y[p][j][la]; with one output column tile the ERIs are
        // sliced inside the GEMM (gathered once), else through bf16 planes
        if (gather) {
            sliced_gemm_packed(ctx, d_int2, pairs.p, p0, np, n, rmax.p, B1, Y.p, OutMap{n, n1});
        } else {
            slice_packed(ctx, d_int2, pairs.p, p0, np, n, A);
            sliced_gemm(ctx, A, B1, Y.p, OutMap{n, n1}, false);
        }
        ctx.trace_mark("mp2 step 1");
        if (dense_gather) {  // rows (p, j) -> Z[p][j][b]
            dense_row_max(ctx, Y.p, np * n1, n, n, dmax.p);
            sliced_gemm_dense_gather(ctx, Y.p, np * n1, n, n, dmax.p, B2, Z.p + p0 * nq, OutMap{0, n2});
        } else {
            slice_dense(ctx, Y.p, np * n1, n, n, A, SLICE_TILE_A);
            sliced_gemm(ctx, A, B2, Z.p + p0 * nq, OutMap{0, n2}, false);
        }
        ctx.trace_mark("mp2 step 2");
    }
    // Z^T: one contiguous row of pairs per q, so that the (q, mu) rows of step 3
    // gather from one L2-resident row instead of one cache line per element
    DBuf<double> Zt((size_t)npair * nq, st);
    transpose_device(ctx, Z.p, npair, nq, Zt.p);
    Z.release();
    ctx.trace_mark("mp2 transpose");
    // steps 3-4 over blocks of q
    const int64_t qb = std::max<int64_t>(1, SLICE_BUDGET_ROWS / std::max(n, n1));
    DBuf<double> W((size_t)std::min(qb, nq) * n1 * n, st);
    for (int64_t q0 = 0; q0 < nq; q0 += qb) {
        const int64_t nqb = std::min(qb, nq - q0);
        // rows (q, mu) over nu of Zt[q0 + q][pair(mu, nu)] -> W[q][i][mu]
        if (gather) {
            sympair_row_max(ctx, Zt.p + q0 * npair, npair, nqb, n, rmax.p);
            sliced_gemm_sympair(ctx, Zt.p + q0 * npair, npair, nqb, n, rmax.p, B1, W.p, OutMap{n, n1});
        } else {
            slice_sympair(ctx, Zt.p + q0 * npair, npair, nqb, n, A);
            sliced_gemm(ctx, A, B1, W.p, OutMap{n, n1}, false);
        }
        ctx.trace_mark("mp2 step 3");
        if (dense_gather) {  // rows (q, i) -> T[q][i][a]
            dense_row_max(ctx, W.p, nqb * n1, n, n, dmax.p);
            sliced_gemm_dense_gather(ctx, W.p, nqb * n1, n, n, dmax.p, B2, T + q0 * n1 * n2, OutMap{0, n2});
        } else {
            slice_dense(ctx, W.p, nqb * n1, n, n, A, SLICE_TILE_A);
            sliced_gemm(ctx, A, B2, T + q0 * n1 * n2, OutMap{0, n2}, false);
        }
        ctx.trace_mark("mp2 step 4");
    }
}

// one block per pair i >= j: sum_ab (ia|jb) [2 (ia|jb) - (ib|ja)] / (e_i + e_j - e_a - e_b)
// from T[j][b][i][a] (relative error of each term ~1e-14 from the refined reciprocal).  For fixed (i, j) the v x v block X[b][a] = (ia|jb) has rows
// of consecutive a; (ib|ja) = X[a][b] is its transpose.  32 x 32 tiles of X and of
// the mirrored tile are staged in shared memory with coalesced row reads, so T is
// read with unit stride instead of one scattered element per (ib|ja).
__global__ void __launch_bounds__(256) mp2_pair_energy_kernel(int o, int v, const double* __restrict__ T,
                                                             const double* __restrict__ eps, double* partial)
{
    __shared__ double A[32][33], B[32][33];
    // block p = the pair i >= j (p = i (i + 1) / 2 + j): the (j, i) block holds the
    // same terms with a and b exchanged ((jb|ia) = (ia|jb)), so it counts twice
    const int p = blockIdx.x;
    int i = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
    while (i * (i + 1) / 2 > p) --i;
    while ((i + 1) * (i + 2) / 2 <= p) ++i;
    const int j = p - i * (i + 1) / 2;
    (void)o;
    const double eij = eps[i] + eps[j];
    const int64_t rs = (int64_t)o * v;  // stride between consecutive b (rows of X)
    const double* X = T + ((int64_t)j * v * o + i) * v;  // X[b][a] = X[b * rs + a]
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    double s = 0.0;
    for (int b0 = 0; b0 < v; b0 += 32)
        for (int a0 = 0; a0 < v; a0 += 32) {
            for (int r = ty; r < 32; r += 8) {
                const int b = b0 + r, a = a0 + tx;
                A[r][tx] = (b < v && a < v) ? X[b * rs + a] : 0.0;    // X[b0 + r][a0 + tx]
                const int bb = a0 + r, aa = b0 + tx;
                B[r][tx] = (bb < v && aa < v) ? X[bb * rs + aa] : 0.0;  // X[a0 + r][b0 + tx]
            }
            __syncthreads();
            for (int r = ty; r < 32; r += 8) {
                const int b = b0 + r, a = a0 + tx;
                if (b < v && a < v) {
                    const double x = A[r][tx], y = B[tx][r];  // (ia|jb), (ib|ja)
                    const double d = eij - eps[o + a] - eps[o + b];
                    // 1/d: FP32 reciprocal (24 bits) and one Newton step in FP64
                    // (~48 bits), instead of an FP64 division on the narrow FP64 pipe
                    const double r0 = (double)__frcp_rn((float)d);
                    const double rd = r0 * fma(-d, r0, 2.0);
                    s = fma(x * (2 * x - y), rd, s);
                }
            }
            __syncthreads();
        }
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = (i == j ? 1.0 : 2.0) * sh[0];
}

double mp2_energy_mixed(Context& ctx, int n, const double* d_int2, const double* dC, int o, const double* d_eps)
{
    const int v = n - o;
    if (o <= 0 || v <= 0) return 0.0;
    DBuf<double> T((size_t)o * v * o * v, ctx.stream);
    ao2mo_sliced(ctx, n, d_int2, dC, o, dC + (size_t)n * o, v, T.p);
    const int npairs = o * (o + 1) / 2;
    DBuf<double> part((size_t)npairs, ctx.stream);
    mp2_pair_energy_kernel<<<npairs, 256, 0, ctx.stream>>>(o, v, T.p, d_eps, part.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
    std::vector<double> h((size_t)npairs);
    part.download(h.data(), h.size());
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
    double E = 0;
    for (double x : h) E += x;
    return E;
}

}  // namespace hfgpu
