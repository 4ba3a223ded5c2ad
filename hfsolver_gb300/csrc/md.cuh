// McMurchie-Davidson building blocks shared by the integral kernels.
//
// Conventions (follow hfsolver's basis, src/basis.f90:371-409):
//   * Cartesian components of a shell with angular momentum L are ordered
//     for k = 0..L, for n = 0..k: (l, m, n) = (L-k, k-n, n).
//   * Hermite functions Lambda_{tuv} are indexed independently of L by
//     hidx(t,u,v): grouped by s = t+u+v, then w = u+v, then v.
//   * A primitive pair (a, b) is expanded as
//       c_a c_b exp(-mu R_AB^2) G_a G_b = sum_tuv E^{ab}_{tuv} Lambda_{tuv}(P),
//     with E^{ab}_{tuv} = Ex^{ax bx}_t Ey^{ay by}_u Ez^{az bz}_v and the 1-D
//     coefficients from the recursion of McMurchie & Davidson,
//     J. Comput. Phys. 26, 218 (1978) (Helgaker, Jorgensen, Olsen,
//     "Molecular Electronic-Structure Theory", eqs. 9.5.6-9.5.7).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace hfgpu {

#define HD __host__ __device__ __forceinline__

HD constexpr int ncart(int L) { return (L + 1) * (L + 2) / 2; }
HD constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
HD constexpr int hidx(int t, int u, int v)
{
    return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + (u + v) * (u + v + 1) / 2 + v;
}

struct Cart {
    int l, m, n;
};

// component i of a shell of angular momentum L (reference order)
HD constexpr Cart cart(int L, int i)
{
    int c = 0;
    for (int k = 0; k <= L; ++k)
        for (int n = 0; n <= k; ++n) {
            if (c == i) return Cart{L - k, k - n, n};
            ++c;
        }
    return Cart{0, 0, 0};
}

// number of non-zero Hermite terms of the component pair (ia, ib)
HD constexpr int box(int la, int ia, int lb, int ib)
{
    return (cart(la, ia).l + cart(lb, ib).l + 1) * (cart(la, ia).m + cart(lb, ib).m + 1) *
           (cart(la, ia).n + cart(lb, ib).n + 1);
}

// offset of component pair (ia, ib) in a primitive-pair E record (ia-major)
HD constexpr int eoff(int la, int lb, int ia, int ib)
{
    int s = 0;
    for (int a = 0; a < ncart(la); ++a)
        for (int b = 0; b < ncart(lb); ++b) {
            if (a == ia && b == ib) return s;
            s += box(la, a, lb, b);
        }
    return s;
}

HD constexpr int ne_pair(int la, int lb) { return eoff(la, lb, ncart(la), 0); }

// position of term (t,u,v) inside the box of component pair (ia, ib)
HD constexpr int eterm(int la, int ia, int lb, int ib, int t, int u, int v)
{
    return (t * (cart(la, ia).m + cart(lb, ib).m + 1) + u) * (cart(la, ia).n + cart(lb, ib).n + 1) + v;
}

// Primitive-pair record: [p, Px, Py, Pz, E terms ...]
constexpr int PAIR_HDR = 4;
HD constexpr int pair_stride(int la, int lb) { return PAIR_HDR + ne_pair(la, lb); }

// Pair types with la >= lb, ordered by number of component pairs:
// ss(0) ps(1) ds(2) pp(3) dp(4) dd(5)
HD constexpr int ptype_la(int t) { return t == 0 ? 0 : t == 1 ? 1 : t == 2 ? 2 : t == 3 ? 1 : t == 4 ? 2 : 2; }
HD constexpr int ptype_lb(int t) { return t == 0 ? 0 : t == 1 ? 0 : t == 2 ? 0 : t == 3 ? 1 : t == 4 ? 1 : 2; }
inline int ptype_of(int la, int lb)
{
    if (la < lb) { int t = la; la = lb; lb = t; }
    if (la == 0) return 0;
    if (la == 1) return lb == 0 ? 1 : 3;
    return lb == 0 ? 2 : lb == 1 ? 4 : 5;
}
constexpr int NPTYPE = 6;

// ------------------------------------------------------------- FP64 helpers
#ifdef __CUDACC__
// 1/sqrt(s) for s > 0 in FP64: an FP32 seed refined by two Newton steps
// y <- y (3 - s y^2) / 2, each doubling the number of correct bits.
__device__ __forceinline__ double rsqrt_nr(double s)
{
    double y = (double)rsqrtf((float)s);
    double h = 0.5 * s;
    y = y * fma(-h * y, y, 1.5);
    y = y * fma(-h * y, y, 1.5);
    return y;
}

// R_tuv(p, PC) for t+u+v <= L (Helgaker et al. eqs. 9.9.18-9.9.20), compile-time L
template <int L>
__device__ __forceinline__ void r_ct(double (&R)[nherm(L)], const double (&F)[L + 1], double X, double Y, double Z)
{
    double Rn[L + 1][nherm(L)];
#pragma unroll
    for (int n = 0; n <= L; ++n) Rn[n][0] = F[n];
#pragma unroll
    for (int n = L - 1; n >= 0; --n)
#pragma unroll
        for (int s = 1; s <= L - n; ++s)
#pragma unroll
            for (int t = s; t >= 0; --t)
#pragma unroll
                for (int v = 0; v <= s - t; ++v) {
                    const int u = s - t - v;
                    double r;
                    if (t > 0) {
                        r = X * Rn[n + 1][hidx(t - 1, u, v)];
                        if (t > 1) r = fma((double)(t - 1), Rn[n + 1][hidx(t - 2, u, v)], r);
                    } else if (u > 0) {
                        r = Y * Rn[n + 1][hidx(0, u - 1, v)];
                        if (u > 1) r = fma((double)(u - 1), Rn[n + 1][hidx(0, u - 2, v)], r);
                    } else {
                        r = Z * Rn[n + 1][hidx(0, 0, v - 1)];
                        if (v > 1) r = fma((double)(v - 1), Rn[n + 1][hidx(0, 0, v - 2)], r);
                    }
                    Rn[n][hidx(t, u, v)] = r;
                }
#pragma unroll
    for (int h = 0; h < nherm(L); ++h) R[h] = Rn[0][h];
}
#endif

}  // namespace hfgpu
