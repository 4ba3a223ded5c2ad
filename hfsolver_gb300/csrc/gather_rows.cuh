// Row sources of the gather-fed GEMMs (tcgemm.cu on the tensor cores,
// dgemm_rows.cu in FP64): each maps a row index r of the A operand to the
// elements of that row, gathered straight from where the transform keeps them
// (the packed AO integrals, Z transposed, or a dense row-major matrix), so that
// no unpacked copy of A goes through HBM.
//   row(r)      per-row state, computed once per row
//   at(w, k)    element k of the row
//   live(r)     false for padding rows of blocked layouts (not loaded or stored)
//   out_row(r)  the row's place in the output's row order
//   row_max(r)  the row's largest |element| (upper word), for the sliced GEMM
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace hfgpu {

struct DenseRows {  // row-major rows with stride ld
    const double* p;
    int64_t ld;
    using Row = const double*;
    __device__ Row row(int64_t r) const { return p + r * ld; }
    __device__ double at(Row w, int k) const { return __ldg(w + k); }
};

// dense row-major rows for the gather-fed GEMM (row maxima from dense_row_max)
struct DenseRowsG {
    const double* p;
    int64_t ld;
    const unsigned* rmax;
    using Row = const double*;
    __device__ Row row(int64_t r) const { return p + r * ld; }
    __device__ double at(Row w, int k) const { return __ldg(w + k); }
    __device__ unsigned long long row_max(int64_t r) const { return (unsigned long long)rmax[r] << 32; }
    __device__ bool live(int64_t) const { return true; }
    __device__ int64_t out_row(int64_t r) const { return r; }
};

struct PackedRows {  // rows (pair p, la), k = si of the packed (mu nu|la si), pairs mu >= nu from p0
    const double* ints;
    const int2* pairs;
    int64_t p0;
    int n;
    struct Row {
        int64_t ij, ij_base;  // pair index of (mu, nu) and ij (ij + 1) / 2
        int la;
    };
    __device__ Row row(int64_t r) const
    {
        const int64_t p = r / n;
        const int2 mn = pairs[p0 + p];
        const int64_t ij = (int64_t)mn.x * (mn.x + 1) / 2 + mn.y;
        return Row{ij, ij * (ij + 1) / 2, (int)(r - p * n)};
    }
    __device__ double at(const Row& w, int si) const
    {
        const int c = w.la > si ? w.la : si, d = w.la > si ? si : w.la;
        const int64_t kl = (int64_t)(c * (c + 1) / 2 + d);
        return __ldg(ints + (w.ij >= kl ? w.ij_base + kl : kl * (kl + 1) / 2 + w.ij));
    }
};

// The same rows for the gather-fed GEMM, in 2-D blocks: a warp's 32 rows are 8
// consecutive pairs x 4 consecutive indices la, a 128-row tile 8 pairs x 16
// indices.  For a fixed si, the elements with pair(la, si) > pair p sit in one
// stored row at consecutive p (one 64-byte run per la), and those with
// pair(la, si) <= p in runs over consecutive la or si: about 40% fewer memory
// transactions per load than rows running over la alone.  Rows past the last
// pair or index are dead (not loaded, not stored).
struct PackedRowsBlocked {
    const double* ints;
    const int2* pairs;
    int64_t p0, np;  // pairs[p0 .. p0 + np)
    int n, nlg;      // nlg = ceil(n / 16) index groups
    const unsigned* rmax;  // row maxima (upper word of |x|) of every pair row, [p][la]
    struct Row {
        int ij;          // pair index of (mu, nu) (< 2^31 for n <= 512)
        int64_t ij_base;  // ij (ij + 1) / 2
        int la;
    };
    __device__ void decode(int64_t r, int64_t& p, int& la) const
    {
        const int64_t t = r >> 7;
        const int q = (int)(r & 127), w = q >> 5, l = q & 31;
        p = (t / nlg) * 8 + (l & 7);
        la = (int)(t % nlg) * 16 + w * 4 + (l >> 3);
    }
    __device__ bool live(int64_t r) const
    {
        int64_t p;
        int la;
        decode(r, p, la);
        return p < np && la < n;
    }
    __device__ int64_t out_row(int64_t r) const  // the row's place in p-major order (p n + la)
    {
        int64_t p;
        int la;
        decode(r, p, la);
        return p * n + la;
    }
    __device__ Row row(int64_t r) const
    {
        int64_t p;
        int la;
        decode(r, p, la);
        const int2 mn = pairs[p0 + p];
        const int ij = mn.x * (mn.x + 1) / 2 + mn.y;
        return Row{ij, ((int64_t)ij * (ij + 1)) >> 1, la};
    }
    __device__ unsigned long long row_max(int64_t r) const
    {
        int64_t p;
        int la;
        decode(r, p, la);
        return (unsigned long long)rmax[(p0 + p) * n + la] << 32;
    }
    // 32-bit index arithmetic up to the final address (64-bit compares would run
    // on the FP64 pipe)
    __device__ double at(const Row& w, int si) const
    {
        const int c = max(w.la, si), d = min(w.la, si);
        const int kl = c * (c + 1) / 2 + d;
        return __ldg(ints + (w.ij >= kl ? w.ij_base + kl : (((int64_t)kl * (kl + 1)) >> 1) + w.ij));
    }
};

struct SymPairRows {  // rows (q, mu), k = nu of Zt[q * ldz + pair(mu, nu)] (Z transposed: one row per q)
    const double* Zt;
    int64_t ldz;
    int n;
    const unsigned* rmax = nullptr;  // row maxima (upper word of |x|), [q][mu] (gather GEMM)
    __device__ unsigned long long row_max(int64_t r) const { return (unsigned long long)rmax[r] << 32; }
    __device__ bool live(int64_t) const { return true; }
    __device__ int64_t out_row(int64_t r) const { return r; }
    struct Row {
        const double* z;
        int mu;
    };
    __device__ Row row(int64_t r) const
    {
        const int64_t q = r / n;
        return Row{Zt + q * ldz, (int)(r - q * n)};
    }
    __device__ double at(const Row& w, int nu) const
    {
        const int a = w.mu > nu ? w.mu : nu, b = w.mu > nu ? nu : w.mu;
        return __ldg(w.z + (a * (a + 1) / 2 + b));
    }
};

}  // namespace hfgpu
