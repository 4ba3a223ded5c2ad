"""Write the host check sources for the generated ERI-gradient class bodies.

For every ordered class (bra type TB, ket type TK) one C++ file takes the
generated GradPrim / GradContract specialisations from gen/grad_class_<TB><TK>.cu
and runs them the way grad_kernel.cuh does (all ket chunks of one quartet,
the bra primitive pairs in turn) for a quartet of contracted shells with
random exponents, coefficients, centres and density values.  The analytic
derivatives with respect to the bra's first centre (gA) and, where the class
has it, to both bra centres together (gP) are compared with central finite
differences of sum Gamma (ab|cd) from the reference ERIs of ref.cpp.

    python make_checks.py GEN_DIR OUT_DIR
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "hfsolver_gb300", "csrc"))
from gen_eri import PTYPES, ncart, nherm  # noqa: E402
from gen_grad import grad_ncd  # noqa: E402


def main(gen_dir, out_dir):
    os.makedirs(os.path.join(out_dir, "cls"), exist_ok=True)
    names = []
    for tb in range(6):
        for tk in range(6):
            txt = open(f"{gen_dir}/grad_class_{tb}{tk}.cu").read()
            body = txt[txt.index("namespace hfgpu {") + len("namespace hfgpu {"):txt.index("GradKernelFn grad_kernel_")]
            la, lb = PTYPES[tb]; lc, ld = PTYPES[tk]
            ncdc = grad_ncd(tb, tk); nh1 = nherm(la + lb + 1); ncdt = ncart(lc) * ncart(ld); G = ncdt // ncdc
            L = la + lb + lc + ld
            kinds = (["true"] if tb <= tk else []) + (["false"] if tb >= tk else [])
            src = f'''#include "common.h"
    namespace hfgpu {{
    {body}
    }}
    using namespace hfgpu;
    std::vector<double> ref_block(const Shell&, const Shell&, const Shell&, const Shell&);
    void make_records(const Shell& A, const Shell& B, const Shell& C, const Shell& D, std::vector<double>& gb, std::vector<double>& ek, int& nbp, int& nkp);
    void boys_row(int M, double T, double* F);
    template <int CH> static void prim_all(double* accs, const double* ek, const double* F, double X, double Y, double Z) {{
        if constexpr (CH < {G}) {{
            GradPrim<{tb}, {tk}, CH>::prim(*(double(*)[{ncdc * nh1}])(accs + CH * {ncdc * nh1}), ek, *(const double(*)[{L + 2}])F, X, Y, Z);
            prim_all<CH + 1>(accs, ek, F, X, Y, Z);
        }}
    }}
    template <bool WP> static void kernel(const Shell& A, const Shell& B, const Shell& C, const Shell& D, const double* gam, double* g) {{
        std::vector<double> gb, ek; int nbp, nkp;
        make_records(A, B, C, D, gb, ek, nbp, nkp);
        const int SG = grad_stride({la}, {lb}), SK = pair_stride({lc}, {ld});
        for (int k = 0; k < 6; ++k) g[k] = 0;
        for (int pb = 0; pb < nbp; ++pb) {{
            const double* rb = gb.data() + pb * SG;
            double accs[{G * ncdc * nh1}] = {{0}};
            for (int pk = 0; pk < nkp; ++pk) {{
                const double* rk = ek.data() + pk * SK;
                double p = rb[2], q = rk[0];
                double r = 1.0 / std::sqrt(p + q), alpha = p * q * r * r;
                double X = rb[3] - rk[1], Y = rb[4] - rk[2], Z = rb[5] - rk[3];
                double T = alpha * (X * X + Y * Y + Z * Z);
                double F[{L + 2}];
                boys_row({L + 1}, T, F);
                double s = 1;
                for (int m = 0; m <= {L + 1}; ++m) {{ F[m] *= 34.986836655249725 * r * s; s *= -2 * alpha; }}
                prim_all<0>(accs, rk + PAIR_HDR, F, X, Y, Z);
            }}
            for (int ch = 0; ch < {G}; ++ch)
                for (int s = 0; s < {ncdc}; ++s)
                    GradContract<{tb}, WP>::template run<{ncdc}>(accs + ch * {ncdc * nh1} + s * {nh1}, gam + ch * {ncdc * ncart(la) * ncart(lb)} + s, rb, *(double(*)[6])g);
        }}
    }}
    int check_{tb}{tk}(const Shell& A, const Shell& B, const Shell& C, const Shell& D, unsigned seed) {{
        const int NAB = {ncart(la) * ncart(lb)}, NCDT = {ncdt}, NCDC = {ncdc}, G = {G};
        std::mt19937 rng(seed); std::uniform_real_distribution<double> U(-1, 1);
        std::vector<double> gam(G * NAB * NCDC), Gfull(NAB * NCDT);
        for (int ch = 0; ch < G; ++ch) for (int ab = 0; ab < NAB; ++ab) for (int s = 0; s < NCDC; ++s) {{
            double v = U(rng); gam[ch * NAB * NCDC + ab * NCDC + s] = v; Gfull[ab * NCDT + ch * NCDC + s] = v; }}
        auto energy = [&](const Shell& a, const Shell& b, const Shell& c, const Shell& d) {{
            auto blk = ref_block(a, b, c, d); double e = 0; for (size_t i = 0; i < blk.size(); ++i) e += Gfull[i] * blk[i]; return e; }};
        int bad = 0;
        for (int wp = 0; wp < 2; ++wp) {{
            if (wp == 1 && !{'true' if 'true' in kinds else 'false'}) continue;
            if (wp == 0 && !{'true' if 'false' in kinds else 'false'}) continue;
            double g[6];
            if (wp) {{ {"kernel<true>(A, B, C, D, gam.data(), g);" if "true" in kinds else ""} }}
            else {{ {"kernel<false>(A, B, C, D, gam.data(), g);" if "false" in kinds else ""} }}
            const double h = 1e-4;
            for (int k = 0; k < 3; ++k) {{
                Shell Ap = A, Am = A; Ap.c[k] += h; Am.c[k] -= h;
                double fd = (energy(Ap, B, C, D) - energy(Am, B, C, D)) / (2 * h);
                double err = std::fabs(fd - g[k]) / (1e-6 + std::fabs(fd));
                if (err > 1e-6) {{ printf("class %d%d wp%d dA%d: analytic %.12e fd %.12e\\n", {tb}, {tk}, wp, k, g[k], fd); ++bad; }}
                if (wp) {{
                    Shell Bp = B, Bm = B; Bp.c[k] += h; Bm.c[k] -= h;
                    double fdp = (energy(Ap, Bp, C, D) - energy(Am, Bm, C, D)) / (2 * h);
                    double e2 = std::fabs(fdp - g[3 + k]) / (1e-6 + std::fabs(fdp));
                    if (e2 > 1e-6) {{ printf("class %d%d dP%d: analytic %.12e fd %.12e\\n", {tb}, {tk}, k, g[3 + k], fdp); ++bad; }}
                }}
            }}
        }}
        return bad;
    }}
    '''
            open(os.path.join(out_dir, "cls", f"c{tb}{tk}.cpp"), "w").write(src)
            names.append(f"{tb}{tk}")
    decl = "\n".join(f"int check_{n}(const Shell&, const Shell&, const Shell&, const Shell&, unsigned);" for n in names)
    calls = "\n".join(f"    {{ auto s = shells({n[0]}, {n[1]}); int b = check_{n}(s[0], s[1], s[2], s[3], 7); printf(\"class {n}: %s\\n\", b ? \"FAIL\" : \"ok\"); bad += b; }}" for n in names)
    open(os.path.join(out_dir, "main.cpp"), "w").write(f'''#include "common.h"
    {decl}
    static const int PT[6][2] = {{{{0,0}},{{1,0}},{{2,0}},{{1,1}},{{2,1}},{{2,2}}}};
    static Shell mk(int L, double x, double y, double z, int np, std::mt19937& rng) {{
        std::uniform_real_distribution<double> U(0.3, 2.0);
        Shell s; s.L = L; s.c[0] = x; s.c[1] = y; s.c[2] = z;
        for (int i = 0; i < np; ++i) s.a.push_back(U(rng));
        for (int c = 0; c < hfgpu::ncart(L) * np; ++c) s.co.push_back(U(rng));
        return s;
    }}
    static std::vector<Shell> shells(int tb, int tk) {{
        std::mt19937 rng(tb * 7 + tk);
        return {{mk(PT[tb][0], 0.1, -0.2, 0.3, 2, rng), mk(PT[tb][1], 0.9, 0.4, -0.5, 2, rng),
                 mk(PT[tk][0], -0.6, 1.1, 0.2, 2, rng), mk(PT[tk][1], 0.3, 0.5, 1.2, 1, rng)}};
    }}
    int main() {{ int bad = 0;
    {calls}
        printf("total bad %d\\n", bad); return bad != 0; }}
    ''')


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
