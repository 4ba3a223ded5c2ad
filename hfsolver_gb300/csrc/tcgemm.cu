// FP64-accurate GEMM on the tcgen05 tensor cores (sm_103a) by exact bf16 slicing.
//
// C[r, c] = sum_k A[r, k] B[k, c] for FP64 A and B, as used by the mixed-
// precision AO->MO transform.  Each row of A (and each column of B) is scaled
// by a power of two 2^e so that |x| < 2^e, rounded to a 42-bit fixed-point
// integer and cut into six 7-bit digits d_0..d_5 (x ~ 2^e sum_t d_t 2^{-7(t+1)}),
// stored as bf16 "slice planes" (integers <= 128 are exact in bf16).  This is
// the error-free splitting of Ozaki, Ogita, Oishi and Rump (Numer. Algorithms
// 59, 95 (2012)) with bf16 tensor-core products:
//   * a product of two digits is < 2^14, so a K-sum of one digit pair over
//     K <= 1024 stays below 2^24 and the FP32 tensor-core accumulation is exact;
//   * digit pairs (i, j) with i + j = t share the weight 2^{-7(t+2)} and are
//     accumulated together in TMEM accumulator t (t = 0..5, 21 products);
//     groups t = 0, 1 stay exact for K <= 512, and the rounding of the later
//     groups is below 2^{-24} of terms that are already 2^{-28} smaller;
//   * the epilogue recombines sum_t acc_t 2^{-7(t+2)} exactly in int64 and
//     applies the row and column scales with one FP64 multiply.
// The result matches an FP64 GEMM to about 2^-42 K max|A_r.| max|B_.c| per element.
//
// Kernel: persistent CTAs (128 threads, one per SM) walk the 128 x 64 output
// tiles.  A K step of 32 is one pipeline stage: the 6 A and 6 B slice tiles
// (TMA, 64-byte swizzle, 72 KiB); three stages are in flight.  One thread
// issues the loads and the 21 x 2 tcgen05.mma (M=128, N=64, K=16, BF16 in,
// FP32 out) per step, queueing step k's products before it waits for step
// k-1's to free that stage for step k-1+3.  The next tile's first loads are
// issued before the epilogue reads TMEM.  Every wait on an mbarrier is bounded
// and reports a timeout through an error flag instead of spinning forever.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
#include <type_traits>

#include "internal.h"
#include "gather_rows.cuh"
#include "slice_bits.cuh"
#include "tcgemm.h"

namespace hfgpu {

constexpr int NSL = 6, SL_BITS = 7;
constexpr int BM = 128, BN = 64, BK = 32;
constexpr int STAGES = 3;
constexpr int A_TILE = BM * BK * 2;  // 8 KiB
constexpr int B_TILE = BN * BK * 2;  // 4 KiB
constexpr int STAGE_BYTES = NSL * (A_TILE + B_TILE);  // 72 KiB: the 12 slice tiles of one K step
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 128;
constexpr uint32_t TMEM_COLS = 512;  // 6 accumulators x 64 columns, rounded to a power of two
constexpr int WAIT_SPINS = 1 << 22;

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// bounded wait on an mbarrier phase; false after WAIT_SPINS polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase)
{
    for (int i = 0; i < WAIT_SPINS; ++i) {
        if (mbar_try_wait(bar, phase)) return true;
        if (i > 32) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            su32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(su32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand tile written by TMA with 64-byte swizzle (rows of BK = 32
// bf16): 8-row groups 512 B apart
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;              // leading byte offset (not used by swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;     // stride byte offset
    d |= (uint64_t)1 << 46;              // descriptor version
    d |= (uint64_t)4 << 61;              // 64-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: BF16 x BF16 -> FP32, both K-major, M = 128, N = BN
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void umma_d(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
        "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 2^e for any integer e (0 below the normal range, where the scaled values of
// the transform are far below anything that matters)
__device__ __forceinline__ double pow2(int e)
{
    if (e < -1022) return 0.0;
    if (e > 1023) e = 1023;
    return __longlong_as_double((int64_t)(e + 1023) << 52);
}

static_assert(NSL == SLICE_NSL && SL_BITS == SLICE_BITS, "slice layout shared with slice_bits.cuh");

// RN((double) S) 2^E, from integer fields where the result is a normal double
// (slice_bits.cuh), else on the FP64 unit; identical results either way
__device__ __forceinline__ double scaled_sum_to_double(long long S, int E)
{
    if (E >= -1022 && E <= 1023) {
        bool ok;
        const uint64_t b = scaled_int_to_double_bits(S, E, ok);
        if (ok) return __longlong_as_double((long long)b);
    }
    return (double)S * pow2(E);
}

// two bf16 lanes minus 128 (exact): 0x4300 | d -> d (slice_bits.cuh)
__device__ __forceinline__ uint32_t bf16x2_minus_128(uint32_t w)
{
    uint32_t r;
    asm("sub.rn.bf16x2 %0, %1, %2;" : "=r"(r) : "r"(w), "r"(0x43004300u));
    return r;
}

// ------------------------------------------------------------------ GEMM kernel
__device__ __forceinline__ int64_t out_index(const OutMap& om, int64_t r, int64_t c)
{
    return om.R > 0 ? (r / om.R) * (om.R * om.ld) + c * om.R + (r % om.R) : r * om.ld + c;
}

__global__ void __launch_bounds__(128, 1)
    sliced_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                       int64_t a_rows_pad, int b_rows_pad, int ksteps, const int* __restrict__ ea,
                       const int* __restrict__ eb, int64_t M, int N, double* out, OutMap om, int accumulate,
                       int* err, int64_t ntiles, int ntn)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);  // TMA landed, one per stage
    uint64_t* empty = full + STAGES;                            // products of the stage done
    uint32_t* tslot = (uint32_t*)(empty + STAGES);
    __shared__ int s_ok;
    auto sA = [&](int s, int t) { return smem + s * STAGE_BYTES + t * A_TILE; };
    auto sB = [&](int s, int t) { return smem + s * STAGE_BYTES + NSL * A_TILE + t * B_TILE; };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;

    // thread 0's bookkeeping: the K step whose load is in flight on each stage
    // (-1: none), and the last K step whose products were committed
    int64_t pend[STAGES];
    for (int s = 0; s < STAGES; ++s) pend[s] = -1;
    int64_t last_commit = -1;
    auto load = [&](int64_t g, int64_t m0, int n0, int ks) {
        const int s = (int)(g % STAGES);
        mbar_expect_tx(&full[s], STAGE_BYTES);
#pragma unroll
        for (int t = 0; t < NSL; ++t) {
            tma_load_2d(sA(s, t), &tmA, ks * BK, (int)(t * a_rows_pad + m0), &full[s]);
            tma_load_2d(sB(s, t), &tmB, ks * BK, t * b_rows_pad + n0, &full[s]);
        }
        pend[s] = g;
    };
    const int pro = ksteps < STAGES ? ksteps : STAGES;

    bool ok = true;
    int64_t g0 = 0;  // K steps run by this CTA before the current tile
    int64_t tile = blockIdx.x;
    if (tile < ntiles && threadIdx.x == 0)
        for (int ks = 0; ks < pro; ++ks) load(ks, (tile / ntn) * BM, (int)(tile % ntn) * BN, ks);
    for (; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t m0 = (tile / ntn) * BM;
        const int n0 = (int)(tile % ntn) * BN;
        if (threadIdx.x == 0) {
            // products of step ks are queued before waiting for those of step ks-1,
            // whose stage is then refilled STAGES steps ahead
            for (int ks = 0; ks < ksteps && ok; ++ks) {
                const int64_t g = g0 + ks;
                const int s = (int)(g % STAGES);
                if (!mbar_wait(&full[s], (uint32_t)((g / STAGES) & 1))) {
                    ok = false;
                    break;
                }
                pend[s] = -1;
                fence_after();
#pragma unroll
                for (int i = 0; i < NSL; ++i)
#pragma unroll
                    for (int j = 0; j < NSL - i; ++j) {
                        const uint32_t dt = tmem + (uint32_t)((i + j) * BN);
#pragma unroll
                        for (int kk = 0; kk < BK / 16; ++kk) {
                            const uint64_t ad = sdesc(su32(sA(s, i)) + kk * 32);
                            const uint64_t bd = sdesc(su32(sB(s, j)) + kk * 32);
                            // group t = i + j is first written by (i = 0, j = t) at ks = 0, kk = 0
                            umma(dt, ad, bd, (ks == 0 && i == 0 && kk == 0) ? 0u : 1u);
                        }
                    }
                umma_commit(&empty[s]);
                last_commit = g;
                if (ks >= 1 && ks - 1 + STAGES < ksteps) {
                    const int64_t gp = g - 1;
                    if (!mbar_wait(&empty[gp % STAGES], (uint32_t)((gp / STAGES) & 1))) {
                        ok = false;
                        break;
                    }
                    load(gp + STAGES, m0, n0, ks - 1 + STAGES);
                }
            }
            s_ok = ok;
        }
        __syncthreads();
        ok = s_ok;
        const int64_t glast = g0 + ksteps - 1;
        if (ok) ok = mbar_wait(&empty[glast % STAGES], (uint32_t)((glast / STAGES) & 1));
        ok = __syncthreads_and(ok);
        // every stage is free again: start the next tile's loads before the epilogue
        const int64_t next = tile + gridDim.x;
        if (ok && threadIdx.x == 0 && next < ntiles)
            for (int ks = 0; ks < pro; ++ks) load(glast + 1 + ks, (next / ntn) * BM, (int)(next % ntn) * BN, ks);
        if (ok) {
            fence_after();
            // epilogue: warp w owns TMEM lanes (rows) 32w .. 32w+31
            // Every group sum is an integer-valued FP32 (sums of digit products), so the
            // groups recombine exactly in int64: S = sum_t acc_t 2^{7(NSL-1-t)} < 2^59,
            // and the value is S 2^{-7(NSL+1)} times the row and column scales.
            const int64_t r = m0 + warp * 32 + lane;
            const int er = (r < M) ? ea[r] : 0;
            for (int c0 = 0; c0 < BN && n0 + c0 < N; c0 += 16) {
                long long S[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) S[i] = 0;
#pragma unroll
                for (int t = 0; t < NSL; ++t) {
                    float f[16];
                    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(t * BN + c0), f);
#pragma unroll
                    for (int i = 0; i < 16; ++i)  // |group sum| < 6 K 2^14 < 2^31 for K <= 512
                        S[i] += (long long)__float2int_rn(f[i]) << (SL_BITS * (NSL - 1 - t));
                }
                if (r < M) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int c = n0 + c0 + i;
                        if (c < N) {
                            const double x = scaled_sum_to_double(S[i], er + eb[c] - SL_BITS * (NSL + 1));
                            const int64_t o = out_index(om, r, c);
                            out[o] = accumulate ? out[o] + x : x;
                        }
                    }
                }
            }
        }
        // the epilogue's TMEM reads finish before the next tile's products overwrite it
        fence_before();
        __syncthreads();
        fence_after();
        g0 += ksteps;
    }
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
        if (threadIdx.x == 0) {
            // let copies and products still in flight land before TMEM and shared memory go (bounded)
            for (int s = 0; s < STAGES; ++s)
                if (pend[s] >= 0) mbar_wait(&full[s], (uint32_t)((pend[s] / STAGES) & 1));
            if (last_commit >= 0) mbar_wait(&empty[last_commit % STAGES], (uint32_t)((last_commit / STAGES) & 1));
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// ------------------------------------------------------------------ slicing
// bf16 bit pattern of sign * v for an integer 0 <= v <= 128 (exact: bf16 holds
// 8 significant bits), built with integer operations only
__device__ __forceinline__ uint16_t small_int_bf16(uint32_t v, uint32_t sign)
{
    if (v == 0) return (uint16_t)(sign << 15);
    const int e = 31 - __clz(v);  // 2^e <= v < 2^(e+1), e <= 7
    return (uint16_t)((sign << 15) | ((uint32_t)(127 + e) << 7) | ((v << (7 - e)) & 0x7Fu));
}

// digits of |x| * 2^(42 - e) (rounded), with the sign of x applied, as bf16
// bit patterns: no floating-point instruction at all (GB300 runs 64-bit
// conversions on its narrow FP64 pipe)
__device__ __forceinline__ void digits_bf16(double x, int e, uint16_t (&d)[NSL])
{
    const uint64_t bits = (uint64_t)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    uint64_t Y = 0;
    if (ex != 0) {
        const uint64_t m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        const int sh = ex - 1075 + NSL * SL_BITS - e;  // |x| < 2^e gives sh < -10
        if (sh >= 0)
            Y = m << sh;
        else if (sh > -63)
            Y = (m + (1ull << (-sh - 1))) >> (-sh);
    }
    const uint32_t sgn = (uint32_t)(bits >> 63);
#pragma unroll
    for (int t = 0; t < NSL; ++t) {
        const int shift = SL_BITS * (NSL - 1 - t);
        const uint32_t dig = (uint32_t)(Y >> shift) & (t == 0 ? 0xFFFFFFFFu : ((1u << SL_BITS) - 1));
        d[t] = small_int_bf16(dig, sgn);
    }
}

// row exponent from the bits of the largest |x| of the row: |x| < 2^e for every
// x in the row (0 for an all-zero row)
__device__ __forceinline__ int row_exponent(uint64_t amax_bits)
{
    if (amax_bits == 0) return 0;
    return (int)((amax_bits >> 52) & 0x7FF) - 1022;
}

// One warp per row.  Src::row(r) sets up the row once; element (r, k) is
// Src::at(row, k).
template <class Src>
__global__ void slice_kernel(Src src, int64_t rows, int K, int64_t rows_pad, int K_pad, __nv_bfloat16* planes,
                             int* rexp)
{
    constexpr int KMAX = 16;  // K <= 512
    const int lane = threadIdx.x & 31;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nwarp) {
        const typename Src::Row row = src.row(r);
        double x[KMAX];
        // the largest |x| as an integer compare of the magnitude bits (finite
        // doubles order like their bit patterns), off the FP64 pipe
        unsigned long long amax = 0;
#pragma unroll
        for (int q = 0; q < KMAX; ++q) {
            const int k = lane + 32 * q;
            x[q] = (k < K) ? src.at(row, k) : 0.0;
            const unsigned long long m = (unsigned long long)__double_as_longlong(x[q]) & 0x7FFFFFFFFFFFFFFFull;
            amax = m > amax ? m : amax;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long v = __shfl_xor_sync(0xffffffffu, amax, o);
            amax = v > amax ? v : amax;
        }
        const int e = row_exponent(amax);
        if (lane == 0) rexp[r] = e;
#pragma unroll
        for (int q = 0; q < KMAX; ++q) {
            const int k = lane + 32 * q;
            if (k < K) {
                uint16_t d[NSL];
                digits_bf16(x[q], e, d);
                uint16_t* pl = reinterpret_cast<uint16_t*>(planes);
#pragma unroll
                for (int t = 0; t < NSL; ++t) pl[((int64_t)t * rows_pad + r) * K_pad + k] = d[t];
            }
        }
    }
}

// ------------------------------------------------------------------ gather-fed GEMM
// The same product with the A operand sliced on the fly: instead of writing six
// bf16 planes of A to HBM and reading them back through TMA, the CTA's threads
// gather A's FP64 elements (Src::row / Src::at), cut them into digits and store
// them straight into the stage's shared-memory tiles in the 64-byte-swizzled
// K-major layout the MMA reads (16-byte chunk c of row r at chunk c ^ ((r >> 1) & 3)).
// B still arrives by TMA.  Each tile first takes its rows' exponents (the
// largest magnitude of each row, from the same gathers).
// 512 threads: thread t produces row t % 128, K quarter t / 128 (8 elements, one
// 16-byte chunk per plane) of every stage, fetching the next stage's elements
// before it stores this one; the 16 producer warps share the epilogue (warp w:
// TMEM lanes 32 (w % 4), columns 16 (w / 4) .. +15).  A 17th warp issues the
// B loads (ahead, into every stage already free) and the products, so that no
// producer waits for a stage's other producers.
constexpr int GATHER_PRODUCERS = 512;
constexpr int GATHER_THREADS = GATHER_PRODUCERS + 32;

// Output-tile width and pipeline depth of the gather-fed GEMM: 64 columns with
// three stages, or 80 columns (16 waters: 80 occupied orbitals in one tile, so
// the rows are gathered once) with two stages to stay within shared memory.
template <int GBN_, int GST_>
struct GatherCfg {
    static constexpr int GBN = GBN_, GST = GST_;
    static constexpr int B_T = GBN * BK * 2;
    static constexpr int STAGE = NSL * (A_TILE + B_T);
    static constexpr int SMEM = GST * STAGE + 1024 + 128;
    static constexpr uint32_t IDESC =
        (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(GBN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
    static_assert(GBN % 16 == 0 && NSL * GBN <= (int)TMEM_COLS, "tile width");
};
using Gather64 = GatherCfg<64, 3>;
using Gather80 = GatherCfg<80, 2>;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}

template <class Src, class C>
__global__ void __launch_bounds__(GATHER_THREADS, 1)
    sliced_gemm_gather_kernel(Src src, const __grid_constant__ CUtensorMap tmB,
                              int b_rows_pad, int K, int ksteps, const int* __restrict__ eb, int64_t M, int N,
                              double* out, OutMap om, int* err, int64_t ntiles, int ntn)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + C::GST * C::STAGE);
    uint64_t* empty = full + C::GST;
    uint32_t* tslot = (uint32_t*)(empty + C::GST);
    __shared__ int s_ok;
    constexpr int PARTS = GATHER_PRODUCERS / BM;  // K parts of a stage per row
    __shared__ int s_exp[BM];  // row exponents of the current tile (for the epilogue)
    auto sA = [&](int s, int t) { return smem + s * C::STAGE + t * A_TILE; };
    auto sB = [&](int s, int t) { return smem + s * C::STAGE + NSL * A_TILE + t * C::B_T; };

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int PK = BK / PARTS;              // elements per thread and stage (8: one 16-byte chunk)
    static_assert(PK == 8, "one 16-byte chunk per thread and plane");
    const int prow = tid & (BM - 1), part = tid / BM;
    const bool producer = tid < GATHER_PRODUCERS, issuer = tid == GATHER_PRODUCERS;
    if (tid == 0) {
        for (int s = 0; s < C::GST; ++s) {
            mbar_init(&full[s], GATHER_PRODUCERS + 1);  // every producer + the B expect_tx
            mbar_init(&empty[s], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_ok = 1;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;

    bool ok = true;
    int64_t g0 = 0;
    int64_t last_commit = -1;  // issuer
    int64_t pend_b = -1;       // issuer: last step whose B load was issued
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t m0 = (tile / ntn) * BM;
        const int n0 = (int)(tile % ntn) * C::GBN;
        const int64_t R = m0 + prow;
        const bool live = producer && R < M && src.live(R);
        const typename Src::Row row = src.row(live ? R : 0);
        // the row's exponent from the precomputed row maximum (row_max kernels);
        // the barrier keeps this tile's s_exp writes behind the last epilogue's reads
        const unsigned long long amax = live ? src.row_max(R) : 0ull;
        __syncthreads();
        const int e = row_exponent(amax);
        if (producer && part == 0) s_exp[prow] = e;
        // this thread's 8 elements of step 0, fetched ahead
        double x[PK];
#pragma unroll
        for (int j = 0; j < PK; ++j) {
            const int k = part * PK + j;
            x[j] = (live && k < K) ? src.at(row, k) : 0.0;
        }
        if (issuer) {
            // B loads for every step up to g + GST - 1 whose stage is free (step g's own
            // is waited for), then step g's products once its stage is full
            int64_t next_b = g0;
            const int64_t gend = g0 + ksteps;
            for (int ks = 0; ks < ksteps && ok; ++ks) {
                const int64_t g = g0 + ks;
                while (next_b < gend && next_b < g + C::GST) {
                    const int sl = (int)(next_b % C::GST);
                    if (next_b >= C::GST) {
                        const uint32_t ph = (uint32_t)(((next_b - C::GST) / C::GST) & 1);
                        if (next_b == g) {
                            if (!mbar_wait(&empty[sl], ph)) {
                                ok = false;
                                break;
                            }
                        } else if (!mbar_try_wait(&empty[sl], ph)) {
                            break;
                        }
                    }
                    mbar_expect_tx(&full[sl], NSL * C::B_T);
#pragma unroll
                    for (int t = 0; t < NSL; ++t)
                        tma_load_2d(sB(sl, t), &tmB, (int)(next_b - g0) * BK, t * b_rows_pad + n0, &full[sl]);
                    pend_b = next_b;
                    ++next_b;
                }
                if (!ok) break;
                const int s = (int)(g % C::GST);
                if (!mbar_wait(&full[s], (uint32_t)((g / C::GST) & 1))) {
                    ok = false;
                    break;
                }
                fence_after();
#pragma unroll
                for (int i = 0; i < NSL; ++i)
#pragma unroll
                    for (int jj = 0; jj < NSL - i; ++jj) {
                        const uint32_t dt = tmem + (uint32_t)((i + jj) * C::GBN);
#pragma unroll
                        for (int kk = 0; kk < BK / 16; ++kk) {
                            const uint64_t ad = sdesc(su32(sA(s, i)) + kk * 32);
                            const uint64_t bd = sdesc(su32(sB(s, jj)) + kk * 32);
                            umma_d(dt, ad, bd, C::IDESC, (ks == 0 && i == 0 && kk == 0) ? 0u : 1u);
                        }
                    }
                umma_commit(&empty[s]);
                last_commit = g;
            }
        }
        for (int ks = 0; ks < ksteps && ok && producer; ++ks) {
            const int64_t g = g0 + ks;
            const int s = (int)(g % C::GST);
            if (g >= C::GST && !mbar_wait(&empty[s], (uint32_t)(((g - C::GST) / C::GST) & 1))) {
                ok = false;
                break;
            }
            // two elements per 32-bit word and plane: digit patterns 0x4300 | d, one
            // packed bf16 subtraction of 128, then the signs (slice_bits.cuh)
            uint32_t w[NSL][PK / 2];
#pragma unroll
            for (int j = 0; j < PK; j += 2) {
                const uint64_t b0 = (uint64_t)__double_as_longlong(x[j]), b1 = (uint64_t)__double_as_longlong(x[j + 1]);
                const uint64_t Y0 = scaled_magnitude(b0, e), Y1 = scaled_magnitude(b1, e);
                const uint32_t sw = sign_word(b0, b1);
#pragma unroll
                for (int t = 0; t < NSL; ++t) w[t][j / 2] = bf16x2_minus_128(digit_word(Y0, Y1, t)) ^ sw;
            }
            // the next step's elements are in flight while this one is stored and multiplied
            if (ks + 1 < ksteps) {
#pragma unroll
                for (int j = 0; j < PK; ++j) {
                    const int k = (ks + 1) * BK + part * PK + j;
                    x[j] = (live && k < K) ? src.at(row, k) : 0.0;
                }
            }
            const int c = part ^ ((prow >> 1) & 3);  // 64-byte swizzle: chunk c of row r at c ^ ((r >> 1) & 3)
#pragma unroll
            for (int t = 0; t < NSL; ++t)
                *reinterpret_cast<uint4*>(sA(s, t) + prow * 64 + c * 16) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
            // the tensor core reads shared memory through the async proxy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&full[s]);
        }
        if (!ok) atomicExch(&s_ok, 0);
        __syncthreads();
        ok = s_ok != 0;
        const int64_t glast = g0 + ksteps - 1;
        if (ok) ok = mbar_wait(&empty[glast % C::GST], (uint32_t)((glast / C::GST) & 1));
        ok = __syncthreads_and(ok);
        if (ok && producer) {
            fence_after();
            // warp w: TMEM lanes 32 (w % 4), 16 columns starting at 16 (w / 4)
            const int64_t r = m0 + (warp & 3) * 32 + lane;
            const int er = s_exp[(warp & 3) * 32 + lane];
            for (int c0 = (warp >> 2) * 16; c0 < C::GBN && n0 + c0 < N; c0 += 64) {
                long long S[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) S[i] = 0;
#pragma unroll
                for (int t = 0; t < NSL; ++t) {
                    float f[16];
                    tmem_ld16(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(t * C::GBN + c0), f);
#pragma unroll
                    for (int i = 0; i < 16; ++i) S[i] += (long long)__float2int_rn(f[i]) << (SL_BITS * (NSL - 1 - t));
                }
                if (r < M && src.live(r)) {
                    const int64_t ro = src.out_row(r);
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int c = n0 + c0 + i;
                        if (c < N) out[out_index(om, ro, c)] = scaled_sum_to_double(S[i], er + eb[c] - SL_BITS * (NSL + 1));
                    }
                }
            }
        }
        fence_before();
        __syncthreads();
        fence_after();
        g0 += ksteps;
    }
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
        if (issuer) {
            // B copies and products still in flight land before shared memory and TMEM go (bounded)
            if (pend_b >= 0) mbar_wait(&full[pend_b % C::GST], (uint32_t)((pend_b / C::GST) & 1));
            if (last_commit >= 0) mbar_wait(&empty[last_commit % C::GST], (uint32_t)((last_commit / C::GST) & 1));
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// ------------------------------------------------------------------ host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    HF_CHECK(fn != nullptr, HFGPU_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    return fn;
}

static CUtensorMap make_map(const Sliced& s, int box_rows)
{
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)s.K_pad, (cuuint64_t)(NSL * s.rows_pad)};
    cuuint64_t strides[1] = {(cuuint64_t)s.K_pad * 2};
    cuuint32_t box[2] = {BK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)s.planes.p, dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    HF_CHECK(r == CUDA_SUCCESS, HFGPU_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return m;
}

static int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

void Sliced::alloc(Context& ctx, int64_t r, int k, int row_tile)
{
    HF_CHECK(k >= 1 && k <= 512, HFGPU_ERR_UNSUPPORTED, "sliced GEMM supports 1 <= K <= 512");
    rows = r;
    K = k;
    rows_pad = round_up(r, row_tile);
    K_pad = (int)round_up(k, BK);
    const size_t need = (size_t)NSL * rows_pad * K_pad;
    if (planes.n < need) planes.alloc(need, ctx.stream);
    if (rexp.n < (size_t)rows_pad) rexp.alloc(rows_pad, ctx.stream);
    HF_CUDA(cudaMemsetAsync(planes.p, 0, need * sizeof(__nv_bfloat16), ctx.stream));
}

template <class Src>
static void launch_slice(Context& ctx, const Src& src, Sliced& s)
{
    const int64_t warps = std::min<int64_t>(s.rows, (int64_t)ctx.num_sms * 64);
    const unsigned blocks = (unsigned)std::max<int64_t>(1, (warps * 32 + 255) / 256);
    slice_kernel<Src><<<blocks, 256, 0, ctx.stream>>>(src, s.rows, s.K, s.rows_pad, s.K_pad, s.planes.p, s.rexp.p);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

void slice_dense(Context& ctx, const double* A, int64_t rows, int K, int64_t ld, Sliced& s, int row_tile)
{
    s.alloc(ctx, rows, K, row_tile);
    launch_slice(ctx, DenseRows{A, ld}, s);
}

void slice_packed(Context& ctx, const double* ints, const int2* pairs, int64_t p0, int64_t npairs, int n, Sliced& s)
{
    s.alloc(ctx, npairs * n, n, BM);
    launch_slice(ctx, PackedRows{ints, pairs, p0, n}, s);
}

void slice_sympair(Context& ctx, const double* Zt, int64_t ldz, int64_t nq, int n, Sliced& s)
{
    s.alloc(ctx, nq * n, n, BM);
    launch_slice(ctx, SymPairRows{Zt, ldz, n}, s);
}

void sliced_gemm(Context& ctx, const Sliced& A, const Sliced& B, double* out, OutMap om, bool accumulate)
{
    HF_CHECK(A.K == B.K && A.K_pad == B.K_pad, HFGPU_ERR_INVALID, "sliced GEMM: K mismatch");
    HF_CHECK(B.rows_pad % BN == 0 && A.rows_pad % BM == 0, HFGPU_ERR_INVALID, "sliced GEMM: padding");
    static bool attr = false;
    if (!attr) {
        HF_CUDA(cudaFuncSetAttribute(sliced_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        attr = true;
    }
    const CUtensorMap ta = make_map(A, BM), tb = make_map(B, BN);
    DBuf<int> err(1, ctx.stream);
    err.zero();
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    HF_CUDA(cudaEventRecord(e0, ctx.stream));
    // persistent CTAs, one per SM, walking the output tiles (column tile fastest)
    const int ntn = (int)(B.rows_pad / BN);
    const int64_t ntiles = (A.rows_pad / BM) * ntn;
    HF_CHECK(ntiles > 0, HFGPU_ERR_INVALID, "sliced GEMM: empty");
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, ctx.num_sms);
    sliced_gemm_kernel<<<grid, 128, SMEM_BYTES, ctx.stream>>>(ta, tb, A.rows_pad, (int)B.rows_pad, A.K_pad / BK,
                                                               A.rexp.p, B.rexp.p, A.rows, (int)B.rows, out, om,
                                                               accumulate ? 1 : 0, err.p, ntiles, ntn);
    count_launch();
    HF_CUDA(cudaGetLastError());
    HF_CUDA(cudaEventRecord(e1, ctx.stream));
    int h = 0;
    err.download(&h, 1);
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx.stat_tc_ms += ms;
    ctx.stat_tc_flops += 2.0 * (NSL * (NSL + 1) / 2) * (double)A.rows * (double)B.rows * (double)A.K;
    HF_CHECK(h == 0, HFGPU_ERR_CUDA, "sliced GEMM: an mbarrier wait timed out");
}

}  // namespace hfgpu

namespace hfgpu {

template <class Src, class C>
static void gather_gemm_cfg(Context& ctx, const Src& src, int64_t M, int64_t M_rows, int K, const Sliced& B, double* out,
                            OutMap om)
{
    HF_CHECK(K == B.K, HFGPU_ERR_INVALID, "gather GEMM: K mismatch");
    const int ntn = (int)((B.rows + C::GBN - 1) / C::GBN);
    HF_CHECK((int64_t)ntn * C::GBN <= B.rows_pad, HFGPU_ERR_INVALID, "gather GEMM: padding");
    static bool attr = false;
    if (!attr) {
        HF_CUDA(cudaFuncSetAttribute(sliced_gemm_gather_kernel<Src, C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     C::SMEM));
        attr = true;
    }
    const CUtensorMap tb = make_map(B, C::GBN);
    DBuf<int> err(1, ctx.stream);
    err.zero();
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    HF_CUDA(cudaEventRecord(e0, ctx.stream));
    const int64_t ntiles = (M + BM - 1) / BM * ntn;
    HF_CHECK(ntiles > 0, HFGPU_ERR_INVALID, "gather GEMM: empty");
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, ctx.num_sms);
    sliced_gemm_gather_kernel<Src, C><<<grid, GATHER_THREADS, C::SMEM, ctx.stream>>>(
        src, tb, (int)B.rows_pad, K, B.K_pad / BK, B.rexp.p, M, (int)B.rows, out, om, err.p, ntiles, ntn);
    count_launch();
    HF_CUDA(cudaGetLastError());
    HF_CUDA(cudaEventRecord(e1, ctx.stream));
    int h = 0;
    err.download(&h, 1);
    HF_CUDA(cudaStreamSynchronize(ctx.stream));
    float ms = 0;
    HF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx.stat_tc_ms += ms;
    ctx.stat_tc_flops += 2.0 * (NSL * (NSL + 1) / 2) * (double)M_rows * (double)B.rows * (double)K;
    if constexpr (std::is_same_v<Src, PackedRowsBlocked>) {
        ctx.stat_tc_step1_ms += ms;
        ctx.stat_tc_step1_n += 1;
    }
    HF_CHECK(h == 0, HFGPU_ERR_CUDA, "gather GEMM: an mbarrier wait timed out");
}

// widest output tile first: every row is gathered once per column tile
// (M: rows of the launch, dead ones included; M_rows: the live rows, for the flop count)
template <class Src>
static void gather_gemm(Context& ctx, const Src& src, int64_t M, int64_t M_rows, int K, const Sliced& B, double* out,
                        OutMap om)
{
    if (B.rows <= Gather64::GBN)
        gather_gemm_cfg<Src, Gather64>(ctx, src, M, M_rows, K, B, out, om);
    else
        gather_gemm_cfg<Src, Gather80>(ctx, src, M, M_rows, K, B, out, om);
}

// ---- row maxima for the gather-fed GEMM
// A row of the gather GEMM is (pair a, la) over si of M[a][pair(la, si)], or
// (q, mu) over nu of Zt[q][pair(mu, nu)]: the maximum |x| over si is the
// maximum over the elements of the symmetric pair-row a whose pair contains la.
// Only its exponent is used (row_exponent), so the maxima are kept as the upper
// 32 bits of |x| (sign cleared), which order like |x| down to the exponent and
// stay on 32-bit integer instructions (64-bit compares and conversions run on
// this GPU's narrow FP64 pipe).
// Folding a stored row (elements kl = (la, si), la >= si, kl < len) onto basis
// indices: a warp takes one run kl = tri(la) .. tri(la) + la (consecutive si,
// coalesced loads); each element counts for si (shared-memory atomicMax,
// distinct per lane) and, as the run's maximum, for la.
__device__ __forceinline__ unsigned abs_hi(double x) { return (unsigned)__double2hiint(x) & 0x7FFFFFFFu; }
// the same straight from memory: the upper 32-bit word of the element, loaded as an integer
__device__ __forceinline__ unsigned abs_hi_at(const double* p)
{
    return __ldg(reinterpret_cast<const unsigned*>(p) + 1) & 0x7FFFFFFFu;
}

__device__ __forceinline__ unsigned warp_max_u32(unsigned v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// one CTA per stored row a: PACKED rows are the lower triangle of the packed
// integrals (row a = M[a][0 .. a], at a (a + 1) / 2); otherwise rows of length
// len_full at src + a * ld.  out[a * n + idx] = folded maximum.
template <bool PACKED>
__global__ void row_max_tri_kernel(const double* __restrict__ src, int64_t ld, int len_full, int n, unsigned* out)
{
    extern __shared__ unsigned smax32[];
    const int a = blockIdx.x;
    const double* row = PACKED ? src + (int64_t)a * (a + 1) / 2 : src + (int64_t)a * ld;
    const int len = PACKED ? a + 1 : len_full;
    for (int i = threadIdx.x; i < n; i += blockDim.x) smax32[i] = 0u;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int la = warp; la < n; la += nw) {
        const int t0 = la * (la + 1) / 2;
        if (t0 >= len) break;  // later runs start further out
        const int smx = min(len - 1 - t0, la);
        unsigned m = 0u;
        for (int si = lane; si <= smx; si += 32) {
            const unsigned v = abs_hi_at(row + t0 + si);
            atomicMax(&smax32[si], v);
            m = max(m, v);
        }
        m = warp_max_u32(m);
        if (lane == 0) atomicMax(&smax32[la], m);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[(int64_t)a * n + i] = smax32[i];
}

// the column part of the packed rows: M[a][b] = M[b][a] for b > a lives in
// stored row b.  A CTA takes 32 consecutive a (one per lane, so a warp's loads of
// row b are one 256-byte segment); its warps stride over b.  Each element counts
// for both indices of pair b, in shared memory laid out [idx][lane] (padded);
// the block's maxima are merged into out by atomicMax.
__global__ void row_max_cols_kernel(const double* __restrict__ ints, int npair, int n, unsigned* out)
{
    extern __shared__ unsigned smax32[];  // n x 33
    const int a0 = blockIdx.x * 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = threadIdx.x; i < n * 33; i += blockDim.x) smax32[i] = 0u;
    __syncthreads();
    const int a = a0 + lane;
    // the warp's stored rows b = b0, b0 + nw, ...: the pair (la, si) of b and the
    // row's offset b (b + 1) / 2 are carried along by additions (64-bit multiplies
    // and divisions are slow on this GPU)
    int b = a0 + 1 + warp;
    int la = (int)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);
    while (la * (la + 1) / 2 > b) --la;
    while ((la + 1) * (la + 2) / 2 <= b) ++la;
    int si = b - la * (la + 1) / 2;
    const double* rowb = ints + (((int64_t)b * (b + 1)) >> 1);
    for (; b < npair; ) {
        if (a < b) {
            const unsigned v = abs_hi_at(rowb + a);
            atomicMax(&smax32[la * 33 + lane], v);
            atomicMax(&smax32[si * 33 + lane], v);
        }
        // advance by nw: row offset (b + 1) + (b + 2) + ... + (b + nw)
        rowb += (int64_t)nw * b + (nw * (nw + 1)) / 2;
        b += nw;
        si += nw;
        while (si > la) {  // la grows by one for every la + 1 pairs
            si -= la + 1;
            ++la;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n * 32; i += blockDim.x) {
        const int idx = i >> 5, l = i & 31;
        const unsigned v = smax32[idx * 33 + l];
        if (a0 + l < npair && v) atomicMax(out + (int64_t)(a0 + l) * n + idx, v);
    }
}

void packed_row_max(Context& ctx, const double* ints, int n, unsigned* out)
{
    const int npair = n * (n + 1) / 2;
    row_max_tri_kernel<true><<<(unsigned)npair, 256, n * sizeof(unsigned), ctx.stream>>>(ints, 0, 0, n, out);
    count_launch();
    HF_CUDA(cudaGetLastError());
    const size_t smem = (size_t)n * 33 * sizeof(unsigned);
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(row_max_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    HF_CHECK(smem <= 200 * 1024, HFGPU_ERR_UNSUPPORTED, "row maxima: basis too large");
    row_max_cols_kernel<<<(unsigned)((npair + 31) / 32), 1024, smem, ctx.stream>>>(ints, npair, n, out);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

void sympair_row_max(Context& ctx, const double* Zt, int64_t ldz, int64_t nq, int n, unsigned* out)
{
    const int npair = n * (n + 1) / 2;
    row_max_tri_kernel<false><<<(unsigned)nq, 256, n * sizeof(unsigned), ctx.stream>>>(Zt, ldz, npair, n, out);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

// one warp per row: the upper word of max |x| over the row's K elements
__global__ void dense_row_max_kernel(const double* __restrict__ A, int64_t rows, int K, int64_t ld, unsigned* out)
{
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= rows) return;
    const double* row = A + r * ld;
    unsigned m = 0u;
    for (int k = lane; k < K; k += 32) m = max(m, abs_hi_at(row + k));
    m = warp_max_u32(m);
    if (lane == 0) out[r] = m;
}

void dense_row_max(Context& ctx, const double* A, int64_t rows, int K, int64_t ld, unsigned* out)
{
    dense_row_max_kernel<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, ctx.stream>>>(A, rows, K, ld, out);
    count_launch();
    HF_CUDA(cudaGetLastError());
}

void sliced_gemm_dense_gather(Context& ctx, const double* A, int64_t rows, int K, int64_t ld, const unsigned* rmax,
                              const Sliced& B, double* out, OutMap om)
{
    const DenseRowsG src{A, ld, rmax};
    gather_gemm(ctx, src, rows, rows, K, B, out, om);
}

void sliced_gemm_packed(Context& ctx, const double* ints, const int2* pairs, int64_t p0, int64_t npairs, int n,
                        const unsigned* rmax, const Sliced& B, double* out, OutMap om)
{
    const int nlg = (n + 15) / 16;
    const PackedRowsBlocked src{ints, pairs, p0, npairs, n, nlg, rmax};
    gather_gemm(ctx, src, (npairs + 7) / 8 * nlg * 128, npairs * n, n, B, out, om);
}

void sliced_gemm_sympair(Context& ctx, const double* Zt, int64_t ldz, int64_t nq, int n, const unsigned* rmax,
                         const Sliced& B, double* out, OutMap om)
{
    SymPairRows src{Zt, ldz, n};
    src.rmax = rmax;
    gather_gemm(ctx, src, nq * n, nq * n, n, B, out, om);
}

}  // namespace hfgpu
