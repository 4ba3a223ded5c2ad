"""Generate the straight-line bodies of the ERI gradient class kernels.

The two-electron gradient is sum_abcd Gamma_abcd d(ab|cd)/dX over the screened
shell quartets.  One kernel differentiates one pair of a quartet (the "bra"
here) and sums the other pair (the "ket") without differentiating it; the
ket's centres are covered by a second launch with the pairs swapped.  For an
ordered class (bra type TB, ket type TK) this script emits:

  GradPrim<TB, TK, CH>::prim   one primitive quartet, ket component pairs of
      chunk CH: the Hermite integrals R_{tuv} up to order L+1 (scalar
      temporaries) and, for every ket component pair cd of the chunk and every
      bra Hermite index tau with |tau| <= la+lb+1,
          X[cd][tau] += sum_{tau' in box(cd)} (-1)^{|tau'|} E^{cd}_{tau'} R_{tau+tau'},
      i.e. the ket primitives are summed before anything touches the bra.
  GradContract<TB, WITHP>::run   one bra primitive pair and one ket component
      pair: with w_ab = Gamma8_{ab,cd} c_a c_b K_ab,
          gA += w_ab sum_tau dE^{ab}/dA_tau X[tau]
          gP += w_ab sum_tau E^{ab}_tau X[tau + 1_x|y|z]     (WITHP only)
      gP is the derivative with respect to moving both bra centres together
      (d/dA + d/dB: a Hermite shift of the bra product).  The bra sums are
      factorised axis by axis (v first, then u, then t) so that each term of
      the 1-D tables is used once.

The 1-D tables of a bra primitive pair (la >= lb) are laid out by the pair
kernel in grad.cu: after a header of 20 doubles, E_x, E_y, E_z and then the
derivative tables D_x, D_y, D_z, each (la+1)(lb+1)(la+lb+2) doubles indexed
((i (lb+1) + j) (la+lb+2) + t), with D(i, j, t) = 2a E(i+1, j, t) - i E(i-1, j, t).

Usage:  python gen_grad.py [outdir]
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from gen_eri import PTYPES, box, cart, eoff, gen_R, herm_list, hidx, ncart, nherm  # noqa: E402

GR_HDR = 20   # alpha, beta, p, Px, Py, Pz, K_ab, unused, c_a K_ab (6), c_b (6)
XCAP = 48     # accumulators X per thread: ket component pairs per chunk x bra Hermite indices


def grad_ncd(tb, tk):
    la, lb = PTYPES[tb]
    lc, ld = PTYPES[tk]
    nh1 = nherm(la + lb + 1)
    ncdt = ncart(lc) * ncart(ld)
    for n in range(ncdt, 0, -1):
        if ncdt % n == 0 and n * nh1 <= XCAP:
            return n
    return 1


def table_size(la, lb):
    return (la + 1) * (lb + 1) * (la + lb + 2)


def gen_prim(tb, tk, ch):
    la, lb = PTYPES[tb]
    lc, ld = PTYPES[tk]
    L = la + lb + lc + ld
    lab = la + lb
    nh1 = nherm(lab + 1)
    ncdc = grad_ncd(tb, tk)
    lines = [f"template <> struct GradPrim<{tb}, {tk}, {ch}> {{",
             "  __device__ __forceinline__ static void prim(double (&acc)[%d], const double* __restrict__ ek," % (ncdc * nh1),
             "      const double (&F)[%d], double X, double Y, double Z) {" % (L + 2)]
    gen_R(L + 1, lines)
    hp = herm_list(lab + 1)
    for s in range(ncdc):
        icd = ch * ncdc + s
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
            a = s * nh1 + hidx(t, u, v)
            expr = f"acc[{a}]"
            for sgn, ki, hr in terms:
                expr = f"fma({'-' if sgn < 0 else ''}k{ki}, r0_{hr}, {expr})"
            lines.append(f"    acc[{a}] = {expr};")
        lines.append("    }")
    lines.append("  }")
    lines.append("};")
    return "\n".join(lines)


def _sum(pairs):
    """fma chain of (coefficient, value) names"""
    c, v = pairs[0]
    expr = f"{c} * {v}"
    for c, v in pairs[1:]:
        expr = f"fma({c}, {v}, {expr})"
    return expr


def gen_contract(tb, withp):
    la, lb = PTYPES[tb]
    nb = ncart(lb)
    ts = table_size(la, lb)
    tw = la + lb + 2

    def eo(d, i, j, t):
        return GR_HDR + d * ts + (i * (lb + 1) + j) * tw + t

    def do(d, i, j, t):
        return GR_HDR + (3 + d) * ts + (i * (lb + 1) + j) * tw + t

    wp = "true" if withp else "false"
    lines = [f"template <> struct GradContract<{tb}, {wp}> {{",
             "  template <int GS>",
             "  __device__ __forceinline__ static void run(const double* __restrict__ x, const double* __restrict__ gam,",
             "      const double* __restrict__ gb, double (&g)[6]) {"]
    for ab in range(ncart(la) * nb):
        ia, ib = ab // nb, ab % nb
        (ax, ay, az), (bx, by, bz) = cart(la, ia), cart(lb, ib)
        nx, ny, nz = ax + bx, ay + by, az + bz
        lines.append(f"    {{ // bra component pair {ab}")
        lines.append(f"    const double w = gam[{ab} * GS] * __ldg(gb + {8 + ia}) * __ldg(gb + {14 + ib});")
        for t in range(nx + 1):
            lines.append(f"    const double ex{t} = __ldg(gb + {eo(0, ax, bx, t)});")
        for t in range(nx + 2):
            lines.append(f"    const double dx{t} = __ldg(gb + {do(0, ax, bx, t)});")
        for u in range(ny + 1):
            lines.append(f"    const double ey{u} = __ldg(gb + {eo(1, ay, by, u)});")
        for u in range(ny + 2):
            lines.append(f"    const double dy{u} = __ldg(gb + {do(1, ay, by, u)});")
        for v in range(nz + 1):
            lines.append(f"    const double ez{v} = __ldg(gb + {eo(2, az, bz, v)});")
        for v in range(nz + 2):
            lines.append(f"    const double dz{v} = __ldg(gb + {do(2, az, bz, v)});")
        # v sums
        vz = [(t, u) for t in range(nx + 2) for u in range(ny + 1)] + [(t, ny + 1) for t in range(nx + 1)]
        for (t, u) in vz:
            lines.append(f"    const double vz{t}_{u} = {_sum([(f'ez{v}', f'x[{hidx(t, u, v)}]') for v in range(nz + 1)])};")
        for t in range(nx + 1):
            for u in range(ny + 1):
                lines.append(f"    const double vd{t}_{u} = {_sum([(f'dz{v}', f'x[{hidx(t, u, v)}]') for v in range(nz + 2)])};")
                if withp:
                    lines.append(f"    const double v1{t}_{u} = "
                                 f"{_sum([(f'ez{v}', f'x[{hidx(t, u, v + 1)}]') for v in range(nz + 1)])};")
        # u sums
        for t in range(nx + 2):
            lines.append(f"    const double wy{t} = {_sum([(f'ey{u}', f'vz{t}_{u}') for u in range(ny + 1)])};")
        for t in range(nx + 1):
            lines.append(f"    const double wd{t} = {_sum([(f'dy{u}', f'vz{t}_{u}') for u in range(ny + 2)])};")
            lines.append(f"    const double wz{t} = {_sum([(f'ey{u}', f'vd{t}_{u}') for u in range(ny + 1)])};")
            if withp:
                lines.append(f"    const double w1{t} = {_sum([(f'ey{u}', f'vz{t}_{u + 1}') for u in range(ny + 1)])};")
                lines.append(f"    const double wv{t} = {_sum([(f'ey{u}', f'v1{t}_{u}') for u in range(ny + 1)])};")
        # t sums
        lines.append(f"    g[0] = fma(w, {_sum([(f'dx{t}', f'wy{t}') for t in range(nx + 2)])}, g[0]);")
        lines.append(f"    g[1] = fma(w, {_sum([(f'ex{t}', f'wd{t}') for t in range(nx + 1)])}, g[1]);")
        lines.append(f"    g[2] = fma(w, {_sum([(f'ex{t}', f'wz{t}') for t in range(nx + 1)])}, g[2]);")
        if withp:
            lines.append(f"    g[3] = fma(w, {_sum([(f'ex{t}', f'wy{t + 1}') for t in range(nx + 1)])}, g[3]);")
            lines.append(f"    g[4] = fma(w, {_sum([(f'ex{t}', f'w1{t}') for t in range(nx + 1)])}, g[4]);")
            lines.append(f"    g[5] = fma(w, {_sum([(f'ex{t}', f'wv{t}') for t in range(nx + 1)])}, g[5]);")
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
        for tk in range(6):
            la, lb = PTYPES[tb]
            lc, ld = PTYPES[tk]
            G = ncart(lc) * ncart(ld) // grad_ncd(tb, tk)
            body = [gen_prim(tb, tk, ch) for ch in range(G)]
            # the bra-side launch of class (tb, tk) (tb <= tk) also moves the bra
            # pair as a whole; the swapped launch (tb > tk, or tb == tk) does not
            kinds = []
            if tb <= tk:
                kinds.append("true")
            if tb >= tk:
                kinds.append("false")
            contract = [gen_contract(tb, k == "true") for k in kinds]
            name = f"grad_class_{tb}{tk}.cu"
            txt = [
                "// Generated by gen_grad.py: do not edit.",
                '#include "../grad_kernel.cuh"',
                "namespace hfgpu {",
                *contract,
                *body,
                f"GradKernelFn grad_kernel_{tb}{tk}(bool withp) {{ return select_grad_kernel<{tb}, {tk}>(withp); }}",
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
