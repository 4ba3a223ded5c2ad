// Host-side basis construction.
//
// build_basis() follows hfsolver's src/basis.f90: the 6-31G** table
// (read_basis, :143-249), one shell per table entry on each atom (get_basis,
// :275-344), Cartesian components in get_cartesian_shell order (:371-409),
// each primitive normalised per component (norm_prim, :93-98) and contractions
// with more than one primitive renormalised (norm_contr, fix_normalization,
// :100-132, :346-369).  The normalisation arithmetic is kept in the reference's
// order, including the factor 2**(2*(l+m+n)+1.5) of norm_prim, which the
// reference evaluates in default (single) precision because the literal 1.5
// has no kind suffix; the coefficients therefore equal the reference's bit for
// bit and so do the integrals built from them.
//
// basis_from_functions() turns a function list in the reference's C-driver
// layout (src/qc.h) back into shells for the shell-based kernels.
#include <cmath>
#include <map>

#include "basis_631gss.h"
#include "internal.h"
#include "md.cuh"

namespace hfgpu {

static const double PI = 3.1415926535897932384626433832795;  // src/constants.f90:12

static double fact2(int n) { return n <= 1 ? 1.0 : n * fact2(n - 2); }

static double norm_prim(int l, int m, int n, double a)
{
    double two_pow = (double)(float)std::ldexp(1.4142135623730951, 2 * (l + m + n) + 1);
    return std::sqrt(two_pow * std::pow(a, l + m + n + 1.5) / fact2(2 * l - 1) / fact2(2 * m - 1) /
                     fact2(2 * n - 1) / std::pow(PI, 1.5));
}

static double norm_contr(int l, int m, int n, const double* a, const double* cu, int np)
{
    double L_ = l + m + n;
    double S = 0;
    for (int i = 0; i < np; i++)
        for (int j = 0; j < np; j++) S = S + cu[i] * cu[j] / std::pow(a[i] + a[j], L_ + 3.0 / 2);
    return 1 / std::pow(PI, 3.0 / 4) *
           std::sqrt(std::pow(2.0, L_) / fact2(2 * l - 1) / fact2(2 * m - 1) / fact2(2 * n - 1)) /
           std::sqrt(S);
}

int Basis::max_l() const
{
    int m = 0;
    for (auto& s : shells) m = s.L > m ? s.L : m;
    return m;
}

int basis_size(int natoms, const int* atno)
{
    int n = 0;
    for (int i = 0; i < natoms; i++) {
        int z = atno[i];
        if (z < 1 || z > HFGPU_BASIS_ZMAX || k631_nshell[z] == 0) return 0;
        for (int s = k631_shell0[z]; s < k631_shell0[z] + k631_nshell[z]; s++)
            n += ncart(k631_shell_l[s]);
    }
    return n;
}

Basis build_basis(int natoms, const int* atno, const double* xyz)
{
    HF_CHECK(natoms >= 1, HFGPU_ERR_INVALID, "natoms must be >= 1");
    Basis b;
    int f = 0;
    for (int i = 0; i < natoms; i++) {
        int z = atno[i];
        HF_CHECK(z >= 1 && z <= HFGPU_BASIS_ZMAX && k631_nshell[z] > 0, HFGPU_ERR_INVALID,
                 "read_basis: atom Z=" + std::to_string(z) + " not found");
        for (int k = 0; k < 3; k++)
            HF_CHECK(std::isfinite(xyz[3 * i + k]), HFGPU_ERR_INVALID, "non-finite coordinate");
        for (int s = k631_shell0[z]; s < k631_shell0[z] + k631_nshell[z]; s++) {
            Shell sh;
            sh.L = k631_shell_l[s];
            HF_CHECK(sh.L <= 2, HFGPU_ERR_UNSUPPORTED, "angular momentum above d is not supported");
            sh.nprim = k631_shell_nprim[s];
            sh.atom = i;
            sh.x = xyz[3 * i];
            sh.y = xyz[3 * i + 1];
            sh.z = xyz[3 * i + 2];
            sh.prim0 = (int)b.alpha.size();
            sh.coef0 = (int)b.coef.size();
            sh.cfn0 = (int)b.comp_fn.size();
            const double* al = k631_alpha + k631_shell_prim0[s];
            const double* co = k631_coef + k631_shell_prim0[s];
            for (int p = 0; p < sh.nprim; p++) b.alpha.push_back(al[p]);
            for (int c = 0; c < ncart(sh.L); c++) {
                Cart cc = cart(sh.L, c);
                std::vector<double> cu(sh.nprim);
                for (int p = 0; p < sh.nprim; p++) cu[p] = co[p] * norm_prim(cc.l, cc.m, cc.n, al[p]);
                if (sh.nprim > 1) {
                    double nn = norm_contr(cc.l, cc.m, cc.n, al, cu.data(), sh.nprim);
                    for (auto& v : cu) v = v * nn;
                }
                for (double v : cu) b.coef.push_back(v);
                b.comp_fn.push_back(f++);
            }
            b.shells.push_back(sh);
        }
    }
    b.nbf = f;
    return b;
}

Basis basis_from_functions(int nbf, const int* nprim, const int* istart, const double* xc,
                           const double* yc, const double* zc, const int* lp, const int* mp,
                           const int* np, int n2, const double* coef, const double* alpha)
{
    HF_CHECK(nbf >= 1, HFGPU_ERR_INVALID, "nbf must be >= 1");
    for (int i = 0; i < nbf; i++) {
        HF_CHECK(nprim[i] >= 1 && istart[i] >= 0 && istart[i] + nprim[i] <= n2, HFGPU_ERR_INVALID,
                 "nprim/istart out of range for function " + std::to_string(i));
        HF_CHECK(lp[i] >= 0 && mp[i] >= 0 && np[i] >= 0, HFGPU_ERR_INVALID, "negative power");
        HF_CHECK(lp[i] + mp[i] + np[i] <= 2, HFGPU_ERR_UNSUPPORTED,
                 "angular momentum above d is not supported");
        HF_CHECK(std::isfinite(xc[i]) && std::isfinite(yc[i]) && std::isfinite(zc[i]),
                 HFGPU_ERR_INVALID, "non-finite centre");
    }
    Basis b;
    b.nbf = nbf;
    auto same_prims = [&](int i, int j) {
        if (nprim[i] != nprim[j] || xc[i] != xc[j] || yc[i] != yc[j] || zc[i] != zc[j]) return false;
        for (int k = 0; k < nprim[i]; k++)
            if (alpha[istart[i] + k] != alpha[istart[j] + k]) return false;
        return true;
    };
    int i = 0;
    while (i < nbf) {
        int L = lp[i] + mp[i] + np[i];
        int nc = ncart(L);
        // the next nc functions form a complete shell in any component order?
        std::vector<int> fmap(nc, -1);
        bool whole = i + nc <= nbf;
        for (int j = i; whole && j < i + nc; j++) {
            if (lp[j] + mp[j] + np[j] != L || !same_prims(i, j)) { whole = false; break; }
            int c = -1;
            for (int k = 0; k < nc; k++) {
                Cart cc = cart(L, k);
                if (cc.l == lp[j] && cc.m == mp[j] && cc.n == np[j]) c = k;
            }
            if (c < 0 || fmap[c] >= 0) { whole = false; break; }
            fmap[c] = j;
        }
        if (!whole) {  // one function alone; the other components are absent
            std::fill(fmap.begin(), fmap.end(), -1);
            for (int k = 0; k < nc; k++) {
                Cart cc = cart(L, k);
                if (cc.l == lp[i] && cc.m == mp[i] && cc.n == np[i]) fmap[k] = i;
            }
        }
        Shell sh;
        sh.L = L;
        sh.nprim = nprim[i];
        sh.x = xc[i];
        sh.y = yc[i];
        sh.z = zc[i];
        sh.prim0 = (int)b.alpha.size();
        sh.coef0 = (int)b.coef.size();
        sh.cfn0 = (int)b.comp_fn.size();
        for (int k = 0; k < sh.nprim; k++) b.alpha.push_back(alpha[istart[i] + k]);
        for (int c = 0; c < nc; c++) {
            int f = fmap[c];
            for (int k = 0; k < sh.nprim; k++) b.coef.push_back(f >= 0 ? coef[istart[f] + k] : 0.0);
            b.comp_fn.push_back(f);
        }
        b.shells.push_back(sh);
        i += whole ? nc : 1;
    }
    return b;
}

}  // namespace hfgpu
