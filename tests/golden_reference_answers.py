"""Known answers asserted by hfsolver's own tests for the molecular GTO path.

Each entry: atomic numbers, geometry (bohr), SCF mixing alpha, the occupied count
the test passes to mbpt2, and the asserted values with their tolerances, each
with its source line in src/tests/.  gf = (1-based orbital, pole, tolerance,
line) of find_pole_diag with Nelec/2 occupied, Nscf = 200, tolE = 1e-10.  Nscf = 40, tolE = 1e-10, tolP = 1e-8
throughout (test_gaussians_molecules.f90:20-23, test_gaussians_atoms.f90:20-23).
"""
ANG2BOHR = 1 / 0.529177249
_a = 0.62558332 * ANG2BOHR

CASES = {
    # test_gaussians_molecules.f90
    "H2": dict(atno=[1, 1], xyz=[[0, 0, 0], [0, 0, 1.4]], alpha=1.0, nocc_mp2=1,
               etot=(-1.13128434, 1e-7, ":42"), e2=(-0.0263, 6e-5, ":48"),
               e3=(-0.00551598, 1e-8, ":52"), lam=[(0, -0.595, 6e-4, ":44")],
               gf=(1, -0.59832340, 1e-8, ":55")),
    "N2": dict(atno=[7, 7], xyz=[[0, 0, 0], [0, 0, 2.074]], alpha=1.0, nocc_mp2=None,
               etot=(-108.94268654, 1e-8, ":66"),
               lam=[(4, -0.630, 6e-4, ":68"), (5, -0.612, 6e-4, ":69"), (6, -0.612, 6e-4, ":70")]),
    "CO": dict(atno=[8, 6], xyz=[[0, 0, 0], [0, 0, 2.132]], alpha=0.8, nocc_mp2=None,
               etot=(-112.73732121, 1e-8, ":79"),
               lam=[(5, -0.633, 6e-4, ":81"), (6, -0.548, 6e-4, ":82")]),
    "CH4_1": dict(atno=[6, 1, 1, 1, 1],
                  xyz=[[0, 0, 0], [2.05, 0, 0], [-0.683292, 1.932773, 0],
                       [-0.683292, -0.966387, -1.673831], [-0.683292, -0.966387, 1.673831]],
                  alpha=1.0, nocc_mp2=5, etot=(-40.20170036, 1e-8, ":106"),
                  e2=(-0.16815509, 1e-7, ":114"), e3=(-0.01819243, 1e-7, ":116"),
                  lam=[(4, -0.545, 6e-4, ":109"), (4, -0.54451008, 1e-8, ":110")],
                  gf=(5, -0.51384473, 1e-8, ":119")),
    "CH4_2": dict(atno=[6, 1, 1, 1, 1],
                  xyz=[[0, 0, 0], [_a, -_a, _a], [-_a, _a, _a], [_a, _a, -_a], [-_a, -_a, -_a]],
                  alpha=1.0, nocc_mp2=5, etot=(-40.20170480, 1e-8, ":137"),
                  e2=(-0.16814994, 1e-6, ":139"), lam=[]),
    "NH3": dict(atno=[7, 1, 1, 1],
                xyz=[[0, 0, 0], [1.913, 0, 0], [-0.548761, 1.832602, 0],
                     [-0.548761, -0.916301, -1.587080]],
                alpha=1.0, nocc_mp2=None, etot=(-56.19457246, 1e-8, ":156"),
                lam=[(4, -0.41491598, 1e-8, ":158")], gf=(5, -0.35357570, 1e-8, ":161")),
    "H2O": dict(atno=[8, 1, 1], xyz=[[0, 0, 0], [1.809, 0, 0], [-0.453549, 1.751221, 0]],
                alpha=1.0, nocc_mp2=5, etot=(-76.02315869, 1e-8, ":183"),
                e2=(-0.19925995, 1e-6, ":189"), e3=(-0.00611895, 1e-6, ":191"),
                lam=[(4, -0.497, 6e-4, ":186")], gf=(5, -0.40499448, 1e-8, ":194")),
    "FH": dict(atno=[9, 1], xyz=[[0, 0, 0], [1.733, 0, 0]], alpha=1.0, nocc_mp2=None,
               etot=(-100.01134814, 1e-8, ":209"),
               lam=[(3, -0.627, 6e-4, ":211"), (4, -0.627, 6e-4, ":212")],
               gf=(5, -0.51894290, 2e-8, ":215")),
    # test_gaussians_atoms.f90
    "He": dict(atno=[2], xyz=[[0, 0, 0]], alpha=1.0, nocc_mp2=1,
               etot=(-2.8551604262, 1e-10, ":41"), e2=(-0.02547703, 1e-6, ":46"), lam=[]),
    "Be": dict(atno=[4], xyz=[[0, 0, 0]], alpha=1.0, nocc_mp2=2,
               etot=(-14.56694436, 1e-8, ":68"), e2=(-0.02950068, 1e-6, ":72"), lam=[]),
    "Ne": dict(atno=[10], xyz=[[0, 0, 0]], alpha=1.0, nocc_mp2=5,
               etot=(-128.4744065196, 1e-10, ":93"), e2=(-0.15176955, 1e-6, ":97"), lam=[]),
    "Mg": dict(atno=[12], xyz=[[0, 0, 0]], alpha=1.0, nocc_mp2=6,
               etot=(-199.59561092, 1e-8, ":117"), e2=(-0.02846287, 1e-6, ":120"), lam=[]),
    # Ar: the test passes Nelec = 12 to mbpt2 although the SCF has 18 electrons
    # (test_gaussians_atoms.f90:131); the asserted E2 pins that 6-orbital sum.
    "Ar": dict(atno=[18], xyz=[[0, 0, 0]], alpha=1.0, nocc_mp2=6,
               etot=(-526.77374492, 1e-8, ":140"), e2=(-0.06205272, 1e-6, ":143"), lam=[]),
}
