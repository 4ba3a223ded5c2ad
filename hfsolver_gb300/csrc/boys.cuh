// Boys function F_m(T) = int_0^1 u^(2m) exp(-T u^2) du on the GPU.
//
// Same quantity as hfsolver's Fm (src/special_functions.f90:189-248), computed
// the GPU way, from the mathematics:
//   * 0 <= T < BOYS_TMAX: Taylor expansion about the nearest grid point
//     T_k = k h (h = 1/16, |d| <= 1/32), using dF_m/dT = -F_{m+1}:
//         F_M(T) = sum_{j<8} F_{M+j}(T_k) (-d)^j / j!,
//     e^{-T} = e^{-T_k} sum_{j<8} (-d)^j / j!, then the downward recursion
//     F_m = (2T F_{m+1} + e^{-T}) / (2m+1)  (Shavitt's eq. 24).  Truncation
//     error <= (1/32)^8/8! ~ 2e-17 relative.
//   * T >= BOYS_TMAX: F_0 = sqrt(pi/T)/2 (erf(sqrt T) = 1 to < 1e-22) and the
//     upward recursion F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T); here e^{-T}
//     contributes < 1e-11 relative, so an FP32 exponential is exact enough.
// The grid values F_m(T_k) are made on the host in extended precision
// (boys_table.cpp) from the convergent series
//     F_m(T) = e^{-T} sum_i (2T)^i / ((2m+1)(2m+3)...(2m+2i+1)).
#pragma once
#include <cuda_runtime.h>

#include "md.cuh"

namespace hfgpu {

constexpr int BOYS_MMAX = 12;                    // largest m a kernel may ask for
constexpr int BOYS_NTAYLOR = 8;                  // Taylor terms
constexpr int BOYS_NCOL = BOYS_MMAX + BOYS_NTAYLOR;  // F_0 .. F_{MMAX+7}
constexpr int BOYS_STRIDE = BOYS_NCOL + 1;       // + e^{-T_k}
constexpr double BOYS_H = 1.0 / 16.0;
constexpr double BOYS_TMAX = 50.0;
constexpr int BOYS_NROW = 801;                   // T_k = k/16, k = 0..800

#ifdef __CUDACC__
// F[0..M] = pref * F_m(T) * s^m  (s = -2 alpha for the Hermite R integrals)
template <int M>
__device__ __forceinline__ void boys_scaled(double T, double pref, double s, const double* __restrict__ tab,
                                            double (&F)[M + 1])
{
    static_assert(M <= BOYS_MMAX, "Boys order beyond table");
    if (T < BOYS_TMAX) {
        int k = __double2int_rn(T * 16.0);
        double d = (double)k * BOYS_H - T;  // -(T - T_k)
        const double* row = tab + k * BOYS_STRIDE;
        double w[BOYS_NTAYLOR];
        w[0] = 1.0;
#pragma unroll
        for (int j = 1; j < BOYS_NTAYLOR; ++j) w[j] = w[j - 1] * d * (1.0 / j);
        double fm = 0.0, ex = 0.0;
#pragma unroll
        for (int j = BOYS_NTAYLOR - 1; j >= 0; --j) {
            fm = fma(__ldg(row + M + j), w[j], fm);
            ex += w[j];
        }
        double e = ex * __ldg(row + BOYS_NCOL);
        F[M] = fm;
#pragma unroll
        for (int m = M - 1; m >= 0; --m) F[m] = fma(2.0 * T, F[m + 1], e) * (1.0 / (2 * m + 1));
        double sc = pref;
#pragma unroll
        for (int m = 0; m <= M; ++m) {
            F[m] *= sc;
            sc *= s;
        }
    } else {
        double r = rsqrt_nr(T);
        double e = (T < 103.0) ? (double)expf(-(float)T) : 0.0;
        double inv2t = 0.5 * r * r;
        double f = 0.88622692545275801364 * r;  // sqrt(pi)/2 / sqrt(T)
        double sc = pref;
        F[0] = f * sc;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            f = fma((double)(2 * m + 1), f, -e) * inv2t;
            sc *= s;
            F[m + 1] = f * sc;
        }
    }
}

#endif

// Host: build the table (BOYS_NROW x BOYS_STRIDE doubles).
void boys_make_table(double* tab);

}  // namespace hfgpu
