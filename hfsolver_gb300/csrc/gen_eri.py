"""Generate the straight-line bodies of the ERI class kernels.

For every quartet class (bra pair type <= ket pair type over ss, ps, ds, pp,
dp, dd) and every ket chunk, emit one device function that adds the
contribution of a single primitive quartet to the thread's accumulators:

  1. Boys values F_n scaled by 2 pi^{5/2}/sqrt(p+q) (-2 alpha)^n,
  2. the Hermite integrals R_{tuv} by the McMurchie-Davidson recursion, as
     scalar temporaries (one per auxiliary order and index),
  3. for each ket component pair cd of the chunk and each bra Hermite index tuv:
        x = sum_{t'u'v' in box(cd)} (-1)^{t'+u'+v'} E^{cd}_{t'u'v'} R_{t+t',u+u',v+v'}
     and acc[ab][cd] += E^{ab}_{tuv} x for the bra component pairs ab whose
     Hermite box contains tuv.
Only non-zero Hermite terms appear, every index is a literal, so the compiler
has nothing left to fold.  The output is written to gen/ next to this file.

Usage:  python gen_eri.py [outdir]
"""
import os
import sys


def ncart(L):
    return (L + 1) * (L + 2) // 2


def nherm(L):
    return (L + 1) * (L + 2) * (L + 3) // 6


def cart(L, i):
    c = 0
    for k in range(L + 1):
        for n in range(k + 1):
            if c == i:
                return (L - k, k - n, n)
            c += 1
    raise ValueError


def hidx(t, u, v):
    s, w = t + u + v, u + v
    return s * (s + 1) * (s + 2) // 6 + w * (w + 1) // 2 + v


def herm_list(L):
    out = []
    for s in range(L + 1):
        for t in range(s, -1, -1):
            for v in range(0, s - t + 1):
                out.append((t, s - t - v, v))
    # ordered so that position == hidx
    out.sort(key=lambda x: hidx(*x))
    return out


PTYPES = [(0, 0), (1, 0), (2, 0), (1, 1), (2, 1), (2, 2)]  # ss ps ds pp dp dd


def box(la, ia, lb, ib):
    a, b = cart(la, ia), cart(lb, ib)
    return (a[0] + b[0] + 1, a[1] + b[1] + 1, a[2] + b[2] + 1)


def eoff(la, lb, ia, ib):
    s = 0
    for x in range(ncart(la)):
        for y in range(ncart(lb)):
            if (x, y) == (ia, ib):
                return s
            bx, by, bz = box(la, x, lb, y)
            s += bx * by * bz
    return s


def ne_pair(la, lb):
    return eoff(la, lb, ncart(la), 0)


def pick_ncd(nab, ncd):
    for n in range(ncd, 0, -1):
        if ncd % n == 0 and nab * n <= 36:
            return n
    return 1


def gen_R(L, lines):
    """R^{(0)}_{tuv} for t+u+v <= L as scalars r0_<h>; level-n temporaries r<n>_<h>."""
    lines.append("    // Hermite integrals R_{tuv}, McMurchie-Davidson recursion")
    for n in range(L + 1):
        lines.append(f"    const double r{n}_0 = F[{n}];")
    for n in range(L - 1, -1, -1):
        for s in range(1, L - n + 1):
            for (t, u, v) in [x for x in herm_list(s) if sum(x) == s]:
                h = hidx(t, u, v)
                if t > 0:
                    a, k, prev2 = "X", t - 1, (hidx(t - 2, u, v) if t > 1 else None)
                    prev1 = hidx(t - 1, u, v)
                elif u > 0:
                    a, k, prev2 = "Y", u - 1, (hidx(t, u - 2, v) if u > 1 else None)
                    prev1 = hidx(t, u - 1, v)
                else:
                    a, k, prev2 = "Z", v - 1, (hidx(t, u, v - 2) if v > 1 else None)
                    prev1 = hidx(t, u, v - 1)
                expr = f"{a} * r{n + 1}_{prev1}"
                if prev2 is not None:
                    if k == 1:
                        expr = f"{expr} + r{n + 1}_{prev2}"
                    else:
                        expr = f"fma({float(k)}, r{n + 1}_{prev2}, {expr})"
                lines.append(f"    const double r{n}_{h} = {expr};")


def gen_body(tb, tk, ch):
    la, lb = PTYPES[tb]
    lc, ld = PTYPES[tk]
    L = la + lb + lc + ld
    lp = la + lb
    nab = ncart(la) * ncart(lb)
    ncdt = ncart(lc) * ncart(ld)
    ncd = pick_ncd(nab, ncdt)
    lines = []
    lines.append(f"template <> struct EriBody<{tb}, {tk}, {ch}> {{")
    lines.append("  __device__ __forceinline__ static void prim(double* __restrict__ acc, const double* __restrict__ eb,")
    lines.append("      const double* __restrict__ ek, const double (&F)[%d], double X, double Y, double Z) {" % (L + 1))
    gen_R(L, lines)
    hp = herm_list(lp)
    for s in range(ncd):
        icd = ch * ncd + s
        ic, id_ = icd // ncart(ld), icd % ncart(ld)
        bx, by, bz = box(lc, ic, ld, id_)
        k0 = eoff(lc, ld, ic, id_)
        lines.append(f"    {{ // ket component pair {icd}")
        for i in range(bx * by * bz):
            lines.append(f"    const double k{i} = __ldg(ek + {k0 + i});")
        for (t, u, v) in hp:
            terms = []
            for tt in range(bx):
                for uu in range(by):
                    for vv in range(bz):
                        ki = (tt * by + uu) * bz + vv
                        sgn = -1 if (tt + uu + vv) % 2 else 1
                        terms.append((sgn, ki, hidx(t + tt, u + uu, v + vv)))
            sgn, ki, hr = terms[0]
            expr = f"{'-' if sgn < 0 else ''}k{ki} * r0_{hr}"
            for sgn, ki, hr in terms[1:]:
                expr = f"fma({'-' if sgn < 0 else ''}k{ki}, r0_{hr}, {expr})"
            lines.append(f"    {{ const double x = {expr};")
            for ab in range(nab):
                ia, ib = ab // ncart(lb), ab % ncart(lb)
                ba = box(la, ia, lb, ib)
                if t < ba[0] and u < ba[1] and v < ba[2]:
                    off = eoff(la, lb, ia, ib) + (t * ba[1] + u) * ba[2] + v
                    a = ab * ncd + s
                    lines.append(f"      acc[{a}] = fma(__ldg(eb + {off}), x, acc[{a}]);")
            lines.append("    }")
        lines.append("    }")
    lines.append("  }")
    lines.append("};")
    return "\n".join(lines)


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "gen")
    os.makedirs(out, exist_ok=True)
    names = []
    for tb in range(6):
        for tk in range(tb, 6):
            la, lb = PTYPES[tb]
            lc, ld = PTYPES[tk]
            nab = ncart(la) * ncart(lb)
            ncdt = ncart(lc) * ncart(ld)
            G = ncdt // pick_ncd(nab, ncdt)
            body = [gen_body(tb, tk, ch) for ch in range(G)]
            name = f"eri_class_{tb}{tk}.cu"
            txt = [
                "// Generated by gen_eri.py: do not edit.",
                '#include "../eri_kernel.cuh"',
                "namespace hfgpu {",
                *body,
                f"KernelFn eri_kernel_{tb}{tk}(int mode) {{ return select_kernel<{tb}, {tk}>(mode); }}",
                "}  // namespace hfgpu",
                "",
            ]
            path = os.path.join(out, name)
            new = "\n".join(txt)
            if not (os.path.exists(path) and open(path).read() == new):
                with open(path, "w") as f:
                    f.write(new)
            names.append(name)
    print("\n".join(names))


if __name__ == "__main__":
    main()
