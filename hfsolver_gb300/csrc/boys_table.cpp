// Host-side generation of the Boys-function grid used by boys.cuh.
// F_m(T_k) for T_k = k/16 is summed in extended precision from the series
//   F_m(T) = e^{-T} sum_{i>=0} (2T)^i / ((2m+1)(2m+3)...(2m+2i+1))
// at the top order m = BOYS_NCOL-1 (all terms positive, no cancellation), and
// the lower orders follow from the stable downward recursion
//   F_m = (2T F_{m+1} + e^{-T}) / (2m+1).
#include <cmath>

#include "boys.cuh"

namespace hfgpu {

void boys_make_table(double* tab)
{
    const int mtop = BOYS_NCOL - 1;
    for (int k = 0; k < BOYS_NROW; ++k) {
        long double T = (long double)k / 16.0L;
        long double ex = expl(-T);
        long double term = 1.0L / (2 * mtop + 1), sum = term;
        for (int i = 1; i < 4000; ++i) {
            term = term * (2 * T) / (2 * mtop + 2 * i + 1);
            sum += term;
            if (term < sum * 1e-24L) break;
        }
        long double F[BOYS_NCOL];
        F[mtop] = sum * ex;
        for (int m = mtop - 1; m >= 0; --m) F[m] = (2 * T * F[m + 1] + ex) / (2 * m + 1);
        for (int m = 0; m < BOYS_NCOL; ++m) tab[k * BOYS_STRIDE + m] = (double)F[m];
        tab[k * BOYS_STRIDE + BOYS_NCOL] = (double)ex;
    }
}

}  // namespace hfgpu
