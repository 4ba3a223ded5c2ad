// Exactly sliced FP64 GEMM on tcgen05 tensor cores (tcgemm.cu).
#pragma once
#include <cuda_bf16.h>

#include "internal.h"

namespace hfgpu {

// Output placement: element (r, c) goes to r*ld + c (R == 0), or, with R > 0,
// to (r/R)*(R*ld) + c*R + r%R (the rows transposed within blocks of R).
struct OutMap {
    int64_t R;
    int64_t ld;
};

// A matrix cut into six bf16 planes of 7-bit digits plus one power-of-two
// exponent per row; rows and K padded to the tile sizes.
struct Sliced {
    DBuf<__nv_bfloat16> planes;
    DBuf<int> rexp;
    int64_t rows = 0, rows_pad = 0;
    int K = 0, K_pad = 0;
    void alloc(Context& ctx, int64_t rows, int K, int row_tile);
};

constexpr int SLICE_TILE_A = 128, SLICE_TILE_B = 64;

// rows of a row-major FP64 matrix (stride ld)
void slice_dense(Context& ctx, const double* A, int64_t rows, int K, int64_t ld, Sliced& s, int row_tile);
// rows (pair p, la) over si of the packed (mu nu|la si), pairs[p0 .. p0+npairs)
void slice_packed(Context& ctx, const double* ints, const int2* pairs, int64_t p0, int64_t npairs, int n, Sliced& s);
// rows (q, mu), q < nq, over nu of Zt[q * ldz + pair(mu, nu)]
void slice_sympair(Context& ctx, const double* Zt, int64_t ldz, int64_t nq, int n, Sliced& s);
// out (+)= A B^T for slices A (M x K) and B (N x K)
void sliced_gemm(Context& ctx, const Sliced& A, const Sliced& B, double* out, OutMap om, bool accumulate);
// out = A B^T with A's rows gathered and sliced inside the GEMM (no A planes in
// HBM): rows (pair p, la) over si of the packed (mu nu|la si) ...
// (rmax: the rows' maxima from packed_row_max, for all pairs) ...
void sliced_gemm_packed(Context& ctx, const double* ints, const int2* pairs, int64_t p0, int64_t npairs, int n,
                        const unsigned* rmax, const Sliced& B, double* out, OutMap om);
// ... or rows (q, mu), q < nq, over nu of Zt[q * ldz + pair(mu, nu)] (rmax from
// sympair_row_max for these nq rows)
void sliced_gemm_sympair(Context& ctx, const double* Zt, int64_t ldz, int64_t nq, int n, const unsigned* rmax,
                         const Sliced& B, double* out, OutMap om);
// max |x| of every gather row, as the upper 32 bits of |x| (enough for its
// exponent): packed integrals, rows (pair p, la) of all n (n + 1) / 2 pairs ->
// out[p * n + la]; Zt rows (q, mu) -> out[q * n + mu]
void packed_row_max(Context& ctx, const double* ints, int n, unsigned* out);
// dense row-major rows (rows x K, stride ld): their maxima, and the gather-fed GEMM
// over them (no A planes in HBM; B may span several 64/80-column tiles)
void dense_row_max(Context& ctx, const double* A, int64_t rows, int K, int64_t ld, unsigned* out);
void sliced_gemm_dense_gather(Context& ctx, const double* A, int64_t rows, int K, int64_t ld, const unsigned* rmax,
                              const Sliced& B, double* out, OutMap om);
void sympair_row_max(Context& ctx, const double* Zt, int64_t ldz, int64_t nq, int n, unsigned* out);
// out[c][r] = in[r][c] for a rows x cols row-major FP64 matrix (mp2_mixed.cu)
void transpose_device(Context& ctx, const double* in, int64_t rows, int64_t cols, double* out);

}  // namespace hfgpu
