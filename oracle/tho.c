/*
 * ORACLE — test infrastructure only.  Nothing in the product links or calls this
 * file; tests/, the smoke check and bench.py's CPU-baseline leg use it as the
 * checker.
 *
 * CPU restatement of hfsolver's Gaussian integral code (src/cints.c and
 * src/qc.c, PyQuante-derived), which evaluates every Cartesian primitive
 * integral with the closed formulas of Taketa, Huzinaga and O-ohata,
 * J. Phys. Soc. Japan 21, 2313 (1966) ("THO"):
 *   - electron repulsion: THO eq. 2.22, one Cartesian primitive quartet at a time
 *     (cints.c:103-183), contracted over primitives (cints.c:72-101);
 *   - overlap (THO 2.12, cints.c:212-244), kinetic (cints.c:186-210) and nuclear
 *     attraction (THO 2.18/3.1, cints.c:246-307);
 *   - the drivers getS/getT/getV/getInts over contracted functions (qc.c:6-131)
 *     and the 8-fold packed index (cints.c:327-347).
 * The arithmetic is kept in the reference's order (libm pow/exp/sqrt, the same
 * factor order in every product) so results agree with the reference to the
 * last bits.  Differences from the reference, none of which change a value:
 * no heap allocation per primitive, the fB factors of eq. 2.22 are tabulated
 * once per quartet, packed indices are 64-bit, and the contracted ERI loop runs
 * in parallel over i with OpenMP when compiled with -fopenmp.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int oracle_boys(int maxm, double t, double *F);

#define NFAC 100
static double FAC[NFAC];

__attribute__((constructor)) static void fac_setup(void)
{
    FAC[0] = 1;
    for (int i = 1; i < NFAC; i++) FAC[i] = i * FAC[i - 1];
}

/* integer-valued factorial ratios, as int like the reference (exact here) */
static inline int ratio2(int a, int b) { return (int)(FAC[a] / FAC[b] / FAC[a - 2 * b]); }
static inline int choose(int a, int b) { return (int)(FAC[a] / (FAC[b] * FAC[a - b])); }
static int dfact(int n) { return n <= 1 ? 1 : n * dfact(n - 2); }

static inline double d2(double x1, double y1, double z1, double x2, double y2, double z2)
{
    return (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2) + (z1 - z2) * (z1 - z2);
}

static inline double centre(double a, double xa, double b, double xb)
{
    return (a * xa + b * xb) / (a + b);
}

/* coefficient of x^s in (x + xpa)^ia (x + xpb)^ib  (cints.c:318-325) */
static double binpre(int s, int ia, int ib, double xpa, double xpb)
{
    double acc = 0.;
    for (int t = 0; t < s + 1; t++)
        if (s - ia <= t && t <= ib)
            acc += choose(ia, s - t) * choose(ib, t) * pow(xpa, ia - s + t) * pow(xpb, ib - t);
    return acc;
}

/* ------------------------------------------------------------------ ERI -- */

#define MAXB 24 /* l1+l2+l3+l4 + 1 for up to g functions */

/* one Cartesian direction of THO eq. 2.22: B[I], I = 0..l1+l2+l3+l4 */
static void tho_B(int l1, int l2, int l3, int l4, double p, double a, double b,
                  double q, double c, double d, double g1, double g2, double delta,
                  double *B)
{
    int nb = l1 + l2 + l3 + l4 + 1;
    double f1[MAXB][MAXB / 2 + 1], f2[MAXB][MAXB / 2 + 1];
    for (int i = 0; i < nb; i++) B[i] = 0.;
    for (int i1 = 0; i1 < l1 + l2 + 1; i1++)
        for (int r1 = 0; r1 < i1 / 2 + 1; r1++)
            f1[i1][r1] = binpre(i1, l1, l2, p - a, p - b) * (ratio2(i1, r1) * pow(4 * g1, r1 - i1));
    for (int i2 = 0; i2 < l3 + l4 + 1; i2++)
        for (int r2 = 0; r2 < i2 / 2 + 1; r2++)
            f2[i2][r2] = binpre(i2, l3, l4, q - c, q - d) * (ratio2(i2, r2) * pow(4 * g2, r2 - i2));
    for (int i1 = 0; i1 < l1 + l2 + 1; i1++)
        for (int i2 = 0; i2 < l3 + l4 + 1; i2++)
            for (int r1 = 0; r1 < i1 / 2 + 1; r1++)
                for (int r2 = 0; r2 < i2 / 2 + 1; r2++)
                    for (int u = 0; u < (i1 + i2) / 2 - r1 - r2 + 1; u++) {
                        int e = i1 + i2 - 2 * (r1 + r2);
                        double v = f1[i1][r1] * pow(-1, i2) * f2[i2][r2] * pow(-1, u) *
                                   ratio2(e, u) * pow(q - p, e - 2 * u) / pow(delta, e - u);
                        B[e - u] = B[e - u] + v;
                    }
}

double oracle_eri_prim(double xa, double ya, double za, int la, int ma, int na, double aa,
                       double xb, double yb, double zb, int lb, int mb, int nb, double ab,
                       double xc, double yc, double zc, int lc, int mc, int nc, double ac,
                       double xd, double yd, double zd, int ld, int md, int nd, double ad)
{
    double Bx[MAXB], By[MAXB], Bz[MAXB], F[3 * MAXB];
    double rab2 = d2(xa, ya, za, xb, yb, zb);
    double rcd2 = d2(xc, yc, zc, xd, yd, zd);
    double xp = centre(aa, xa, ab, xb), yp = centre(aa, ya, ab, yb), zp = centre(aa, za, ab, zb);
    double xq = centre(ac, xc, ad, xd), yq = centre(ac, yc, ad, yd), zq = centre(ac, zc, ad, zd);
    double rpq2 = d2(xp, yp, zp, xq, yq, zq);
    double g1 = aa + ab, g2 = ac + ad;
    double delta = (1. / g1 + 1. / g2) / 4.;
    tho_B(la, lb, lc, ld, xp, xa, xb, xq, xc, xd, g1, g2, delta, Bx);
    tho_B(ma, mb, mc, md, yp, ya, yb, yq, yc, yd, g1, g2, delta, By);
    tho_B(na, nb, nc, nd, zp, za, zb, zq, zc, zd, g1, g2, delta, Bz);
    oracle_boys(la + lb + lc + ld + ma + mb + mc + md + na + nb + nc + nd, 0.25 * rpq2 / delta, F);
    double acc = 0.;
    for (int I = 0; I < la + lb + lc + ld + 1; I++)
        for (int J = 0; J < ma + mb + mc + md + 1; J++)
            for (int K = 0; K < na + nb + nc + nd + 1; K++)
                acc += Bx[I] * By[J] * Bz[K] * F[I + J + K];
    return 2. * pow(M_PI, 2.5) / (g1 * g2 * sqrt(g1 + g2)) * exp(-aa * ab * rab2 / g1) *
           exp(-ac * ad * rcd2 / g2) * acc;
}

/* contracted (ij|kl) over basis functions i, j, k, l (cints.c:72-101) */
static double eri_contracted(const int *nprim, const int *istart, const double *xc,
                             const double *yc, const double *zc, const int *lp,
                             const int *mp, const int *np, const double *coef,
                             const double *alpha, int i, int j, int k, int l)
{
    double acc = 0.;
    for (int p = 0; p < nprim[i]; p++)
        for (int q = 0; q < nprim[j]; q++)
            for (int r = 0; r < nprim[k]; r++)
                for (int s = 0; s < nprim[l]; s++) {
                    int ip = istart[i] + p, jp = istart[j] + q, kp = istart[k] + r, lq = istart[l] + s;
                    double v = oracle_eri_prim(
                        xc[i], yc[i], zc[i], lp[i], mp[i], np[i], alpha[ip],
                        xc[j], yc[j], zc[j], lp[j], mp[j], np[j], alpha[jp],
                        xc[k], yc[k], zc[k], lp[k], mp[k], np[k], alpha[kp],
                        xc[l], yc[l], zc[l], lp[l], mp[l], np[l], alpha[lq]);
                    acc += coef[ip] * coef[jp] * coef[kp] * coef[lq] * v;
                }
    return acc;
}

/* 8-fold packed index of (ij|kl), 0-based (cints.c:327-347, 64-bit here) */
int64_t oracle_ijkl(int64_t i, int64_t j, int64_t k, int64_t l)
{
    int64_t t;
    if (i < j) { t = i; i = j; j = t; }
    if (k < l) { t = k; k = l; l = t; }
    int64_t ij = i * (i + 1) / 2 + j, kl = k * (k + 1) / 2 + l;
    if (ij < kl) { t = ij; ij = kl; kl = t; }
    return ij * (ij + 1) / 2 + kl;
}

/* all unique contracted ERIs into the packed array (qc.c:95-131) */
void oracle_getInts(int nbf, const int *nprim, const int *istart, const double *xc,
                    const double *yc, const double *zc, const int *lp, const int *mp,
                    const int *np, int n2, const double *coef, const double *alpha,
                    double *Ints)
{
    (void)n2;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = nbf - 1; i >= 0; i--)
        for (int j = 0; j < i + 1; j++) {
            int64_t ij = (int64_t)i * (i + 1) / 2 + j;
            for (int k = 0; k < nbf; k++)
                for (int l = 0; l < k + 1; l++) {
                    int64_t kl = (int64_t)k * (k + 1) / 2 + l;
                    if (ij >= kl)
                        Ints[oracle_ijkl(i, j, k, l)] = eri_contracted(
                            nprim, istart, xc, yc, zc, lp, mp, np, coef, alpha, i, j, k, l);
                }
        }
}

/* oracle_getInts with quartets left at zero when their Schwarz bound
 * sqrt((ij|ij)) sqrt((kl|kl)) is below thr.  Not a reference routine (the
 * reference computes every quartet): it makes oracle fixtures of 300-400
 * functions affordable.  With thr far below the GPU path's cut (1e-16 against
 * 1e-12) the dropped integrals are below 1e-16 each; the fixture generator
 * checks the screened oracle against the unscreened one at 200 functions.
 * Ints must be zero on entry; Q (nbf(nbf+1)/2 doubles) receives the bounds. */
void oracle_getInts_screened(int nbf, const int *nprim, const int *istart, const double *xc,
                             const double *yc, const double *zc, const int *lp, const int *mp,
                             const int *np, int n2, const double *coef, const double *alpha,
                             double thr, double *Q, double *Ints)
{
    (void)n2;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < nbf; i++)
        for (int j = 0; j <= i; j++) {
            double d = eri_contracted(nprim, istart, xc, yc, zc, lp, mp, np, coef, alpha, i, j, i, j);
            Q[(int64_t)i * (i + 1) / 2 + j] = sqrt(fabs(d));
        }
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = nbf - 1; i >= 0; i--)
        for (int j = 0; j < i + 1; j++) {
            int64_t ij = (int64_t)i * (i + 1) / 2 + j;
            for (int k = 0; k < nbf; k++)
                for (int l = 0; l < k + 1; l++) {
                    int64_t kl = (int64_t)k * (k + 1) / 2 + l;
                    if (ij >= kl && Q[ij] * Q[kl] >= thr)
                        Ints[oracle_ijkl(i, j, k, l)] = eri_contracted(
                            nprim, istart, xc, yc, zc, lp, mp, np, coef, alpha, i, j, k, l);
                }
        }
}

/* out[(nu * n + la) * n + si] = (mu nu|la si) for one mu, from the packed
 * integrals (the semi-direct MP2 of the oracle fixtures unpacks one mu at a
 * time). */
void oracle_unpack_mu(int n, const double *int2, int mu, double *out)
{
#pragma omp parallel for schedule(static)
    for (int nu = 0; nu < n; nu++)
        for (int la = 0; la < n; la++)
            for (int si = 0; si < n; si++)
                out[((int64_t)nu * n + la) * n + si] = int2[oracle_ijkl(mu, nu, la, si)];
}

/* contracted ERIs for an explicit list of function quartets q[4*t..4*t+3] */
void oracle_eri_list(int nbf, const int *nprim, const int *istart, const double *xc,
                     const double *yc, const double *zc, const int *lp, const int *mp,
                     const int *np, const double *coef, const double *alpha, int64_t nq,
                     const int *q, double *out)
{
    (void)nbf;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < nq; t++)
        out[t] = eri_contracted(nprim, istart, xc, yc, zc, lp, mp, np, coef, alpha,
                                q[4 * t], q[4 * t + 1], q[4 * t + 2], q[4 * t + 3]);
}

/* ------------------------------------------------------ one-electron ----- */

static double ovl1d(int l1, int l2, double pax, double pbx, double g)
{
    double acc = 0.;
    for (int i = 0; i < 1 + floor(0.5 * (l1 + l2)); i++)
        acc += binpre(2 * i, l1, l2, pax, pbx) * dfact(2 * i - 1) / pow(2 * g, i);
    return acc;
}

static double ovl_prim(double a1, int l1, int m1, int n1, double xa, double ya, double za,
                       double a2, int l2, int m2, int n2, double xb, double yb, double zb)
{
    double rab2 = d2(xa, ya, za, xb, yb, zb);
    double g = a1 + a2;
    double xp = centre(a1, xa, a2, xb), yp = centre(a1, ya, a2, yb), zp = centre(a1, za, a2, zb);
    double pre = pow(M_PI / g, 1.5) * exp(-a1 * a2 * rab2 / g);
    double wx = ovl1d(l1, l2, xp - xa, xp - xb, g);
    double wy = ovl1d(m1, m2, yp - ya, yp - yb, g);
    double wz = ovl1d(n1, n2, zp - za, zp - zb, g);
    return pre * wx * wy * wz;
}

static double kin_prim(double a1, int l1, int m1, int n1, double xa, double ya, double za,
                       double a2, int l2, int m2, int n2, double xb, double yb, double zb)
{
    double t0 = a2 * (2 * (l2 + m2 + n2) + 3) *
                ovl_prim(a1, l1, m1, n1, xa, ya, za, a2, l2, m2, n2, xb, yb, zb);
    double t1 = -2 * pow(a2, 2) *
                (ovl_prim(a1, l1, m1, n1, xa, ya, za, a2, l2 + 2, m2, n2, xb, yb, zb) +
                 ovl_prim(a1, l1, m1, n1, xa, ya, za, a2, l2, m2 + 2, n2, xb, yb, zb) +
                 ovl_prim(a1, l1, m1, n1, xa, ya, za, a2, l2, m2, n2 + 2, xb, yb, zb));
    double t2 = -0.5 * (l2 * (l2 - 1) * ovl_prim(a1, l1, m1, n1, xa, ya, za, a2, l2 - 2, m2, n2, xb, yb, zb) +
                        m2 * (m2 - 1) * ovl_prim(a1, l1, m1, n1, xa, ya, za, a2, l2, m2 - 2, n2, xb, yb, zb) +
                        n2 * (n2 - 1) * ovl_prim(a1, l1, m1, n1, xa, ya, za, a2, l2, m2, n2 - 2, xb, yb, zb));
    return t0 + t1 + t2;
}

/* one Cartesian direction of THO eq. 2.18: A[I], I = 0..l1+l2 */
static void tho_A(int l1, int l2, double pa, double pb, double cp, double g, double *A)
{
    int n = l1 + l2 + 1;
    for (int i = 0; i < n; i++) A[i] = 0.;
    for (int i = 0; i < n; i++)
        for (int r = 0; r < floor(i / 2) + 1; r++)
            for (int u = 0; u < floor((i - 2 * r) / 2.) + 1; u++) {
                double v = pow(-1, i) * binpre(i, l1, l2, pa, pb) * pow(-1, u) * FAC[i] *
                           pow(cp, i - 2 * r - 2 * u) * pow(0.25 / g, r + u) / FAC[r] / FAC[u] /
                           FAC[i - 2 * r - 2 * u];
                A[i - 2 * r - u] += v;
            }
}

static double nuc_prim(double x1, double y1, double z1, int l1, int m1, int n1, double a1,
                       double x2, double y2, double z2, int l2, int m2, int n2, double a2,
                       double x3, double y3, double z3)
{
    double Ax[MAXB], Ay[MAXB], Az[MAXB], F[3 * MAXB];
    double g = a1 + a2;
    double xp = centre(a1, x1, a2, x2), yp = centre(a1, y1, a2, y2), zp = centre(a1, z1, a2, z2);
    double rab2 = d2(x1, y1, z1, x2, y2, z2);
    double rcp2 = d2(x3, y3, z3, xp, yp, zp);
    tho_A(l1, l2, xp - x1, xp - x2, xp - x3, g, Ax);
    tho_A(m1, m2, yp - y1, yp - y2, yp - y3, g, Ay);
    tho_A(n1, n2, zp - z1, zp - z2, zp - z3, g, Az);
    oracle_boys(l1 + l2 + m1 + m2 + n1 + n2, rcp2 * g, F);
    double acc = 0.;
    for (int I = 0; I < l1 + l2 + 1; I++)
        for (int J = 0; J < m1 + m2 + 1; J++)
            for (int K = 0; K < n1 + n2 + 1; K++)
                acc += Ax[I] * Ay[J] * Az[K] * F[I + J + K];
    return -2 * M_PI / g * exp(-a1 * a2 * rab2 / g) * acc;
}

/* S, T (qc.c:6-58) and V (qc.c:61-93), column-major nbf x nbf */
void oracle_getS(int nbf, const int *nprim, const int *istart, const double *xc,
                 const double *yc, const double *zc, const int *lp, const int *mp,
                 const int *np, int n2, const double *coef, const double *alpha, double *S)
{
    (void)n2;
    for (int j = 0; j < nbf; j++)
        for (int i = 0; i < nbf; i++) {
            S[i + j * nbf] = 0.;
            for (int q = 0; q < nprim[j]; q++) {
                int jj = istart[j] + q;
                for (int p = 0; p < nprim[i]; p++) {
                    int ii = istart[i] + p;
                    S[i + j * nbf] += coef[ii] * coef[jj] *
                                      ovl_prim(alpha[ii], lp[i], mp[i], np[i], xc[i], yc[i], zc[i],
                                               alpha[jj], lp[j], mp[j], np[j], xc[j], yc[j], zc[j]);
                }
            }
        }
}

void oracle_getT(int nbf, const int *nprim, const int *istart, const double *xc,
                 const double *yc, const double *zc, const int *lp, const int *mp,
                 const int *np, int n2, const double *coef, const double *alpha, double *T)
{
    (void)n2;
    for (int j = 0; j < nbf; j++)
        for (int i = 0; i < nbf; i++) {
            T[i + j * nbf] = 0.;
            for (int q = 0; q < nprim[j]; q++) {
                int jj = istart[j] + q;
                for (int p = 0; p < nprim[i]; p++) {
                    int ii = istart[i] + p;
                    T[i + j * nbf] += coef[ii] * coef[jj] *
                                      kin_prim(alpha[ii], lp[i], mp[i], np[i], xc[i], yc[i], zc[i],
                                               alpha[jj], lp[j], mp[j], np[j], xc[j], yc[j], zc[j]);
                }
            }
        }
}

void oracle_getV(int nbf, const int *nprim, const int *istart, const double *xc,
                 const double *yc, const double *zc, const int *lp, const int *mp,
                 const int *np, int n2, const double *coef, const double *alpha, int nat,
                 const int *atno, const double *x, const double *y, const double *z, double *V)
{
    (void)n2;
    for (int j = 0; j < nbf; j++)
        for (int i = 0; i < nbf; i++) {
            V[i + j * nbf] = 0.;
            for (int q = 0; q < nprim[j]; q++) {
                int jj = istart[j] + q;
                for (int p = 0; p < nprim[i]; p++) {
                    int ii = istart[i] + p;
                    for (int a = 0; a < nat; a++)
                        V[i + j * nbf] += coef[ii] * coef[jj] * atno[a] *
                                          nuc_prim(xc[i], yc[i], zc[i], lp[i], mp[i], np[i], alpha[ii],
                                                   xc[j], yc[j], zc[j], lp[j], mp[j], np[j], alpha[jj],
                                                   x[a], y[a], z[a]);
                }
            }
        }
}

/* ------------------------------------------------------------- SCF ------ */

/* G(i,j) = sum_kl P(k,l) [(ij|kl) - 1/2 (il|kj)], scf.f90:39-58 (formG2),
 * column-major n x n, from the packed integrals.  Parallel over j. */
void oracle_formG(int n, const double *P, const double *int2, double *G)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double acc = 0.;
            for (int l = 0; l < n; l++)
                for (int k = 0; k < n; k++) {
                    double tt = int2[oracle_ijkl(i, j, k, l)] - 0.5 * int2[oracle_ijkl(i, l, k, j)];
                    acc += P[k + (int64_t)l * n] * tt;
                }
            G[i + (int64_t)j * n] = acc;
        }
}

/* The same G as oracle_formG, summed in a different order: each unique packed
 * integral (ij|kl) is read once and its eight permutations are scattered into
 * G (J from the (ij) and (kl) pairs, K from the four cross pairs).  n^4/8 reads
 * instead of formG2's 2 n^4 gathers, for oracle SCF runs beyond 200 functions.
 * Per-thread G accumulators are summed at the end.  G is column-major n x n. */
void oracle_formG_scatter(int n, const double *P, const double *int2, double *G)
{
    const int64_t m = (int64_t)n * (n + 1) / 2;
    const int64_t nn = (int64_t)n * n;
    for (int64_t e = 0; e < nn; e++) G[e] = 0.;
#pragma omp parallel
    {
        double *Gt = (double *)calloc((size_t)nn, sizeof(double));
#pragma omp for schedule(dynamic, 16)
        for (int64_t ij = 0; ij < m; ij++) {
            int i = (int)((sqrt(8.0 * (double)ij + 1.0) - 1.0) / 2.0);
            while ((int64_t)i * (i + 1) / 2 > ij) i--;
            while ((int64_t)(i + 1) * (i + 2) / 2 <= ij) i++;
            int j = (int)(ij - (int64_t)i * (i + 1) / 2);
            const double *row = int2 + ij * (ij + 1) / 2;
            int k = 0, l = 0;
            for (int64_t kl = 0; kl <= ij; kl++) {
                double v = row[kl];
                if (v != 0.) {
                    /* weight: each distinct member of the 8-fold orbit once */
                    double w = v;
                    if (i == j) w *= 0.5;
                    if (k == l) w *= 0.5;
                    if (ij == kl) w *= 0.5;
                    /* J: member (x y|z w) adds v P(z,w) to G(x,y) */
                    double pkl = P[k + (int64_t)l * n] + P[l + (int64_t)k * n];
                    double pij = P[i + (int64_t)j * n] + P[j + (int64_t)i * n];
                    Gt[i + (int64_t)j * n] += w * pkl;
                    Gt[j + (int64_t)i * n] += w * pkl;
                    Gt[k + (int64_t)l * n] += w * pij;
                    Gt[l + (int64_t)k * n] += w * pij;
                    /* K: member (x y|z w) adds -v/2 P(z,y) to G(x,w) */
                    double hw = 0.5 * w;
                    Gt[i + (int64_t)l * n] -= hw * P[k + (int64_t)j * n];
                    Gt[j + (int64_t)l * n] -= hw * P[k + (int64_t)i * n];
                    Gt[i + (int64_t)k * n] -= hw * P[l + (int64_t)j * n];
                    Gt[j + (int64_t)k * n] -= hw * P[l + (int64_t)i * n];
                    Gt[k + (int64_t)j * n] -= hw * P[i + (int64_t)l * n];
                    Gt[l + (int64_t)j * n] -= hw * P[i + (int64_t)k * n];
                    Gt[k + (int64_t)i * n] -= hw * P[j + (int64_t)l * n];
                    Gt[l + (int64_t)i * n] -= hw * P[j + (int64_t)k * n];
                }
                if (++l > k) { k++; l = 0; }
            }
        }
#pragma omp critical
        for (int64_t e = 0; e < nn; e++) G[e] += Gt[e];
        free(Gt);
    }
}

/* G(i,j) of formG2 for a list of (i,j) entries only (bounded timing samples of
 * the Fock build at sizes where the full n^4 sweep is too slow). */
void oracle_formG_entries(int n, const double *P, const double *int2, int64_t ne, const int *ij,
                          double *out)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t e = 0; e < ne; e++) {
        int i = ij[2 * e], j = ij[2 * e + 1];
        double acc = 0.;
        for (int l = 0; l < n; l++)
            for (int k = 0; k < n; k++) {
                double tt = int2[oracle_ijkl(i, j, k, l)] - 0.5 * int2[oracle_ijkl(i, l, k, j)];
                acc += P[k + (int64_t)l * n] * tt;
            }
        out[e] = acc;
    }
}
