"""GPU integrals (libhfgpu through the C ABI) against the oracle.

ERIs: |gpu - oracle| <= 1e-12 + 1e-12 |v| per unique integral (FP64 on both
sides; the two use different but exact integral formulas, McMurchie-Davidson
on the GPU and THO in the oracle).  S, T, V: the same bound."""
import numpy as np
import pytest

import hfsolver_gb300 as hf
from tests.golden_reference_answers import CASES
from tests.gpu_common import assert_close, basis_args

pytestmark = pytest.mark.gpu

MOLS = ["H2O", "CH4_1", "NH3", "FH", "Ne", "CO", "Ar"]


@pytest.mark.parametrize("name", MOLS)
def test_eri_packed_matches_oracle(oracle, name):
    c = CASES[name]
    b = oracle.Basis(c["atno"], np.array(c["xyz"], float))
    ref = oracle.getInts(b)
    got = hf.getInts(*basis_args(b))
    assert_close(got, ref, 1e-12, 1e-12, name)


def test_eri_water_dimer_matches_oracle(oracle):
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(2, seed=3)
    b = oracle.Basis(atno, xyz)
    ref = oracle.getInts(b)
    got = hf.getInts(*basis_args(b))
    assert_close(got, ref, 1e-12, 1e-12, "dimer")


@pytest.mark.parametrize("name", ["H2O", "CH4_1", "Ne"])
def test_one_electron_matches_oracle(oracle, name):
    c = CASES[name]
    b = oracle.Basis(c["atno"], np.array(c["xyz"], float))
    args = basis_args(b)
    assert_close(hf.getS(*args), oracle.one_electron(b, "S"), 1e-12, 1e-12, "S")
    assert_close(hf.getT(*args), oracle.one_electron(b, "T"), 1e-12, 1e-12, "T")
    V = hf.getV(*args, b.atno, b.xyz[:, 0], b.xyz[:, 1], b.xyz[:, 2])
    assert_close(V, oracle.one_electron(b, "V"), 1e-11, 1e-12, "V")


def test_getints2_plugin_layout(oracle):
    c = CASES["NH3"]
    b = oracle.Basis(c["atno"], np.array(c["xyz"], float))
    got = hf.getints2(b.nprim, b.istart + 1, b.center.T, b.power.T, b.coef, b.alpha)
    assert_close(got, oracle.getInts(b), 1e-12, 1e-12, "getints2")


def test_function_lists_that_are_not_whole_shells(oracle):
    """The drop-in accepts any function list: components of a shell in another
    order, and functions that do not form a complete shell."""
    c = CASES["H2O"]
    b = oracle.Basis(c["atno"], np.array(c["xyz"], float))
    n = b.n
    rng = np.random.default_rng(1)
    # permute functions within each group of equal centre and nprim, and drop three
    keep = [i for i in range(n) if i not in (3, 11, 20)]
    perm = []
    i = 0
    while i < len(keep):
        j = i
        while (j < len(keep) and np.allclose(b.center[keep[j]], b.center[keep[i]])
               and b.nprim[keep[j]] == b.nprim[keep[i]]):
            j += 1
        block = keep[i:j]
        perm.extend(rng.permutation(block))
        i = j
    perm = np.array(perm)
    nprim = b.nprim[perm]
    coef, alpha, istart = [], [], []
    for f in perm:
        istart.append(len(coef))
        coef.extend(b.coef[b.istart[f]:b.istart[f] + b.nprim[f]])
        alpha.extend(b.alpha[b.istart[f]:b.istart[f] + b.nprim[f]])
    sub = oracle.Basis.__new__(oracle.Basis)
    sub.n = len(perm)
    sub.nprim = np.ascontiguousarray(nprim, dtype=np.int32)
    sub.istart = np.array(istart, dtype=np.int32)
    sub.center = b.center[perm]
    sub.power = np.ascontiguousarray(b.power[perm])
    sub.coef = np.array(coef)
    sub.alpha = np.array(alpha)
    ref = oracle.getInts(sub)
    got = hf.getInts(*basis_args(sub))
    assert_close(got, ref, 1e-12, 1e-12, "permuted")
    assert_close(hf.getS(*basis_args(sub)), oracle.one_electron(sub, "S"), 1e-12, 1e-12, "S permuted")


def test_schwarz_screening_bounds_the_error():
    """Dropping quartets with sqrt((ab|ab)(cd|cd)) < 1e-12 changes E_HF by far
    less than the 1e-10 Ha budget on a spread-out water trimer."""
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(3, box=9.0, seed=5)
    o = dict(tolP=1e-10, tolE=1e-12, diis=True, mp2="none")
    full = hf.rhf(atno, xyz, hf.RHFOptions(**o))
    scr = hf.rhf(atno, xyz, hf.RHFOptions(schwarz=1e-12, **o))
    assert scr["n_quartets"] < full["n_quartets"]
    assert abs(full["Etot"] - scr["Etot"]) < 1e-11
