/*
 * ORACLE — test infrastructure only.  Nothing in the product links or calls this
 * file; tests/, the smoke check and bench.py's CPU-baseline leg use it as the
 * checker.
 *
 * Boys function F_m(t) = int_0^1 u^(2m) exp(-t u^2) du for m = 0..maxm,
 * restated from hfsolver src/special_functions.f90:189-248 (subroutine Fm):
 *   - t <  maxm + 1/2: Shavitt's series for F_maxm, summed until the next term
 *     is below machine epsilon relative to the sum (:223-235), then the downward
 *     recursion F_m = (2 t F_{m+1} + e^{-t}) / (2m + 1) (:237-239);
 *   - otherwise F_0 = 1/2 sqrt(pi/t) erf(sqrt t) and the upward recursion
 *     F_{m+1} = ((2m + 1) F_m - e^{-t}) / (2t) (:241-246).
 * Argument checks follow :218-221 (0 <= maxm <= 500, t >= 0).
 *
 * c_Fm has the C signature that src/cints.c:26 expects from the Fortran
 * binding src/qc.f90:90-95, so the reference's own cints.c links against it.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Fortran epsilon(1._dp) */
#define FORTRAN_DP_EPS 2.220446049250313080847e-16

int oracle_boys(int maxm, double t, double *F)
{
    if (maxm < 0 || maxm > 500) return 1;
    if (!(t >= 0)) return 2;
    if (t < maxm + 0.5) {
        double term = 1.0 / (2 * maxm + 1);
        double s = term;
        int k = 1;
        while (term / s > FORTRAN_DP_EPS) {
            term = term * (2 * t) / (2 * maxm + 2 * k + 1);
            s = s + term;
            k = k + 1;
        }
        F[maxm] = s * exp(-t);
        for (int m = maxm - 1; m >= 0; m--)
            F[m] = (2 * t * F[m + 1] + exp(-t)) / (2 * m + 1);
    } else {
        F[0] = 0.5 * sqrt(M_PI / t) * erf(sqrt(t));
        for (int m = 0; m < maxm; m++)
            F[m + 1] = ((2 * m + 1) * F[m] - exp(-t)) / (2 * t);
    }
    return 0;
}

/* Callback with the reference's calling convention.  Like stop_error in the
 * reference, invalid arguments end the process with exit status 1. */
void c_Fm(int *maxm, double *t, double *F)
{
    int rc = oracle_boys(*maxm, *t, F);
    if (rc) {
        fprintf(stderr, "Fm: %s\n",
                rc == 1 ? "only works for 0 <= m <= 500" : "only works for t >= 0");
        exit(1);
    }
}
