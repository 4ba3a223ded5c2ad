// Host build of the generated ERI-gradient class bodies (gen_grad.py): the
// device qualifiers of md.cuh vanish under a host compiler and __ldg becomes a
// plain load, so GradPrim / GradContract run on the CPU exactly as written.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "md.cuh"
static inline double __ldg(const double* p) { return *p; }
namespace hfgpu {
constexpr int GR_HDR = 20;
inline constexpr int grad_table(int la, int lb) { return (la + 1) * (lb + 1) * (la + lb + 2); }
inline constexpr int grad_stride(int la, int lb) { return GR_HDR + 6 * grad_table(la, lb); }
template <int TB, int TK, int CH>
struct GradPrim;
template <int TB, bool WITHP>
struct GradContract;
}  // namespace hfgpu
// a contracted shell: angular momentum, centre, exponents, coefficients co[component * nprim + primitive]
struct Shell {
    int L;
    double c[3];
    std::vector<double> a;
    std::vector<double> co;
};
