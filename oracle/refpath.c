/*
 * ORACLE — test infrastructure only (the CPU baseline of bench.py).  Nothing in
 * the product links or calls this file.
 *
 * hfsolver's per-molecule algorithm after the integrals, restated in C in the
 * reference's loop order so that its cost can be measured on bounded samples:
 *   - doscf's dense TT precompute, TT(k,l,i,j) = (ij|kl) - 1/2 (il|kj), built
 *     once from the packed integrals (src/scf.f90:84-105);
 *   - formG, G(i,j) = sum(P * TT(:,:,i,j)), every SCF iteration
 *     (src/scf.f90:26-37, called at :109);
 *   - transform_int2's four quarter transforms by dot products
 *     (src/mbpt.f90:32-77);
 *   - term1, the MBPT2 sum with packed-index gathers (src/mbpt2.f90:8-31).
 * Arrays are Fortran-ordered (column-major, 1-based in the reference, 0-based
 * here).  Each routine works on a slab of its outermost loop index so that a
 * caller can time a sample and scale by the loop's length; nthreads > 1 runs
 * the slab's outer loop in parallel with OpenMP (the reference is serial).
 */
#include <stdint.h>

int64_t oracle_ijkl(int64_t i, int64_t j, int64_t k, int64_t l);

/* TT(k, l, i, j) for i in i_list[0..ni) and every j, k, l, stored as
 * TT[((s * n + j) * n + l) * n + k] for the s-th listed i (scf.f90:84-105:
 * loops i, j, k, l with l innermost). */
void refpath_tt_slab(int n, const double *int2, int ni, const int *i_list, double *TT, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) collapse(2)
    for (int s = 0; s < ni; s++)
        for (int j = 0; j < n; j++) {
            const int i = i_list[s];
            double *blk = TT + ((int64_t)s * n + j) * n * n;
            for (int k = 0; k < n; k++)
                for (int l = 0; l < n; l++)
                    blk[(int64_t)l * n + k] = int2[oracle_ijkl(i, j, k, l)] - 0.5 * int2[oracle_ijkl(i, l, k, j)];
        }
}

/* G(i, j) = sum(P * TT(:, :, i, j)) for the slab's ni values of i (scf.f90:26-37);
 * G_slab[s * n + j]. */
void refpath_formG_slab(int n, const double *P, int ni, const double *TT, double *G_slab, int nthreads)
{
    const int64_t nn = (int64_t)n * n;
#pragma omp parallel for schedule(static) num_threads(nthreads) collapse(2)
    for (int s = 0; s < ni; s++)
        for (int j = 0; j < n; j++) {
            const double *blk = TT + ((int64_t)s * n + j) * nn;
            double acc = 0.;
            for (int64_t e = 0; e < nn; e++) acc += P[e] * blk[e];
            G_slab[(int64_t)s * n + j] = acc;
        }
}

/* Step 1, (mu nu|alpha beta) -> (mu nu|k beta), for mu in mu_list
 * (mbpt.f90:32-43): per (nu, beta) gather the n integrals over alpha from the
 * packed array, then n dot products with the columns of C.  Output slab
 * out[((s * n + beta) * n + k) * n + nu] = temp(mu_s, nu, k, beta). */
void refpath_step1(int n, const double *int2, const double *C, int ns, const int *mu_list, double *out,
                   int nthreads)
{
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) collapse(2)
    for (int s = 0; s < ns; s++)
        for (int nu = 0; nu < n; nu++) {
            const int mu = mu_list[s];
            double tempvec[1024];
            for (int beta = 0; beta < n; beta++) {
                for (int alpha = 0; alpha < n; alpha++) tempvec[alpha] = int2[oracle_ijkl(mu, nu, alpha, beta)];
                for (int k = 0; k < n; k++) {
                    const double *ck = C + (int64_t)k * n;
                    double acc = 0.;
                    for (int a = 0; a < n; a++) acc += ck[a] * tempvec[a];
                    out[(((int64_t)s * n + beta) * n + k) * n + nu] = acc;
                }
            }
        }
}

/* Step 2, (mu nu|k beta) -> (i nu|k beta), for nu in the slab (mbpt.f90:45-53):
 * temp(:, nu, k, beta) is a contiguous column over mu in the reference's
 * layout; here T_nu[(s * n + beta) * n + k) * n + mu] holds it for the s-th nu.
 * Output temp2(i, nu, k, beta) as out[((s * n + beta) * n + k) * n + i]. */
void refpath_step2(int n, const double *C, int ns, const double *T_nu, double *out, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) collapse(2)
    for (int s = 0; s < ns; s++)
        for (int beta = 0; beta < n; beta++)
            for (int k = 0; k < n; k++) {
                const double *col = T_nu + (((int64_t)s * n + beta) * n + k) * n;
                for (int i = 0; i < n; i++) {
                    const double *ci = C + (int64_t)i * n;
                    double acc = 0.;
                    for (int m = 0; m < n; m++) acc += ci[m] * col[m];
                    out[(((int64_t)s * n + beta) * n + k) * n + i] = acc;
                }
            }
}

/* Step 3, (i nu|k beta) -> (i nu|k l), l <= k, for one value of i per slab
 * entry (mbpt.f90:55-63).  The reference reads temp2(i, nu, k, :), a vector
 * with a stride of n^3 doubles; here the slab T2[((beta * n + k) * n + nu) *
 * stride + s] keeps the same access pattern (one element per cache line) with
 * stride >= 8 doubles.  Output out[((s * n + l) * n + k) * n + nu]. */
void refpath_step3(int n, const double *C, int ns, int64_t stride, const double *T2, double *out, int nthreads)
{
    const int64_t bstride = (int64_t)n * n * stride;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) collapse(2)
    for (int s = 0; s < ns; s++)
        for (int nu = 0; nu < n; nu++)
            for (int k = 0; k < n; k++) {
                const double *v = T2 + ((int64_t)k * n + nu) * stride + s;
                for (int l = 0; l <= k; l++) {
                    const double *cl = C + (int64_t)l * n;
                    double acc = 0.;
                    for (int b = 0; b < n; b++) acc += cl[b] * v[b * bstride];
                    out[(((int64_t)s * n + l) * n + k) * n + nu] = acc;
                }
            }
}

/* Step 4, (i nu|k l) -> (i j|k l) into the packed MO array, for k in k_list
 * (mbpt.f90:65-77): temp(i, :, k, l) is a row with stride n; T3 holds
 * temp(:, :, k, l) for the slab's (k, l) pairs as T3[((s * n + l) * n + nu) *
 * n + i] (l <= k).  Writes moint2 at the packed index of (i j|k l). */
void refpath_step4(int n, const double *C, int ns, const int *k_list, const double *T3, double *moint2,
                   int nthreads)
{
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int s = 0; s < ns; s++) {
        const int k = k_list[s];
        for (int l = 0; l <= k; l++) {
            const int64_t kl = (int64_t)k * (k + 1) / 2 + l;
            const double *blk = T3 + ((int64_t)s * n + l) * n * n;
            for (int j = 0; j < n; j++) {
                const double *cj = C + (int64_t)j * n;
                for (int i = j; i < n; i++) {
                    const int64_t ij = (int64_t)i * (i + 1) / 2 + j;
                    if (ij < kl) continue;
                    double acc = 0.;
                    for (int nu = 0; nu < n; nu++) acc += cj[nu] * blk[(int64_t)nu * n + i];
                    moint2[oracle_ijkl(i, j, k, l)] = acc;
                }
            }
        }
    }
}

/* term1 (mbpt2.f90:8-31) for the occupied a in a_list: four packed gathers per
 * (a, b, r, s); returns the partial sum over the listed a. */
double refpath_term1(int n, const double *moint2, const double *lam, int nocc, int na, const int *a_list,
                     int nthreads)
{
    double E2 = 0.;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : E2) collapse(2)
    for (int t = 0; t < na; t++)
        for (int b = 0; b < nocc; b++) {
            const int a = a_list[t];
            for (int r = nocc; r < n; r++)
                for (int s = nocc; s < n; s++)
                    E2 += (2. * moint2[oracle_ijkl(a, r, b, s)] * moint2[oracle_ijkl(r, a, s, b)] -
                           1. * moint2[oracle_ijkl(a, r, b, s)] * moint2[oracle_ijkl(s, a, r, b)]) /
                          (-lam[r] - lam[s] + lam[a] + lam[b]);
        }
    return E2;
}

#ifdef _OPENMP
#include <omp.h>
#endif
/* threads OpenMP may use in routines without an explicit count (the ERI list) */
void refpath_set_threads(int nthreads)
{
#ifdef _OPENMP
    omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}
