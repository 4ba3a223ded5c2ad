"""Generate basis_631gss.h, the 6-31G** contraction table compiled into libhfgpu.

The table must hold exactly the numbers hfsolver's `read_basis` reads
(src/basis.f90:143-249, file src/tests/p631ss.txt), so that basis functions,
normalisation and therefore every integral agree with the reference.  Each value
is written with Python's shortest round-trip repr, so a C compiler parses it to
the same double that a list-directed Fortran read of the file produces.

Usage:  python gen_basis_data.py <path to p631ss.txt>   (writes next to this file)
"""
import os
import sys

LCHAR = {"S": 0, "P": 1, "D": 2, "F": 3, "G": 4}


def parse(path):
    toks = open(path).read().split("\n")
    i = 0
    atoms = {}
    while i < len(toks):
        s = toks[i].strip()
        if not s:
            i += 1
            continue
        z = int(s)
        nsh = int(toks[i + 1])
        i += 2
        shells = []
        for _ in range(nsh):
            lch, npr = toks[i].split()
            i += 1
            prims = []
            for _ in range(int(npr)):
                a, c = toks[i].split()
                prims.append((float(a), float(c)))
                i += 1
            shells.append((LCHAR[lch.upper()], prims))
        atoms[z] = shells
    return atoms


def main():
    src = sys.argv[1]
    atoms = parse(src)
    zmax = max(atoms)
    nshell, shell0, sh_l, sh_n, sh_p0, alpha, coef = [], [], [], [], [], [], []
    for z in range(zmax + 1):
        shells = atoms.get(z, [])
        shell0.append(len(sh_l))
        nshell.append(len(shells))
        for l, prims in shells:
            sh_l.append(l)
            sh_n.append(len(prims))
            sh_p0.append(len(alpha))
            for a, c in prims:
                alpha.append(a)
                coef.append(c)

    def arr(name, ctype, vals, fmt):
        body = ",".join(fmt(v) for v in vals)
        return f"static const {ctype} {name}[{len(vals)}] = {{{body}}};\n"

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis_631gss.h")
    with open(out, "w") as f:
        f.write("/* 6-31G** contraction table (Z = 0..%d; Z = 0 is empty).\n" % zmax)
        f.write(" * Generated by gen_basis_data.py from hfsolver's src/tests/p631ss.txt,\n")
        f.write(" * the file read by src/basis.f90:143-249.  Do not edit by hand.\n")
        f.write(" * Coefficients are relative to normalised primitives (basis.f90:20-23). */\n")
        f.write("#pragma once\n")
        f.write("#define HFGPU_BASIS_ZMAX %d\n" % zmax)
        f.write(arr("k631_nshell", "int", nshell, str))
        f.write(arr("k631_shell0", "int", shell0, str))
        f.write(arr("k631_shell_l", "int", sh_l, str))
        f.write(arr("k631_shell_nprim", "int", sh_n, str))
        f.write(arr("k631_shell_prim0", "int", sh_p0, str))
        f.write(arr("k631_alpha", "double", alpha, repr))
        f.write(arr("k631_coef", "double", coef, repr))
    print("wrote", out)


if __name__ == "__main__":
    main()
