"""GPU RHF / transform / MBPT2 against the oracle and the reference's own
known answers.  Tolerances: E_HF 1e-10 Ha and E_MP2 1e-8 Ha against the
oracle on the same inputs; the reference's tolerances (1e-7 .. 1e-10) against
its asserted values."""
import numpy as np
import pytest

import hfsolver_gb300 as hf
from tests.golden_reference_answers import CASES
from tests.gpu_common import assert_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(CASES))
def test_rhf_reference_known_answers(oracle, name):
    c = CASES[name]
    atno, xyz = c["atno"], np.array(c["xyz"], float)
    o = hf.RHFOptions(nscf=40, mix_alpha=c["alpha"], tolE=1e-10, tolP=1e-8, mp2="fp64",
                      mp2_nocc=c["nocc_mp2"] or 0)
    r = hf.rhf(atno, xyz, o, want_orbitals=True)
    val, tol, _ = c["etot"]
    assert abs(r["Etot"] - val) < tol
    for idx, v, t, _ in c["lam"]:
        assert abs(r["lam"][idx] - v) < t
    if "e2" in c:
        val, tol, _ = c["e2"]
        assert abs(r["E2"] - val) < tol
    # the same algorithm as the oracle, step for step: same iteration count
    ref = oracle.rhf_gauss(atno, xyz, nscf=40, alpha=c["alpha"], tolE=1e-10, tolP=1e-8)
    assert r["niter"] == ref["niter"]
    assert abs(r["Etot"] - ref["Etot"]) < 1e-10


def test_single_water_config(oracle):
    """One H2O (0.9572 A, 104.52 deg), 6-31G**, RHF to dP < 1e-10, then MBPT2."""
    from hfsolver_gb300.clusters import water

    atno, xyz = water()
    r = hf.rhf(atno, xyz, hf.RHFOptions(nscf=100, tolP=1e-10, tolE=1e-12))
    ref = oracle.rhf_gauss(atno, xyz, nscf=100, tolE=1e-12, tolP=1e-10)
    e2 = oracle.mbpt2(oracle.transform_int2(ref["int2"], ref["C"]), ref["lam"], 5)
    assert abs(r["Etot"] - ref["Etot"]) < 1e-10
    assert abs(r["E2"] - e2) < 1e-8
    assert r["nbf"] == 25 and r["nocc"] == 5


def test_doscf_dropin(oracle):
    c = CASES["H2O"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    C, P, lam, E0, it = hf.doscf(ref["H"], ref["int2"], ref["S"], 5, 40, 1e-10, 1e-8, 1.0)
    assert it == ref["niter"]
    assert abs(E0 - ref["E0"]) < 1e-10
    assert_close(lam, ref["lam"], 1e-9, 0, "lam")
    assert_close(P, ref["P"], 1e-8, 0, "P")


def test_formG_dropin(oracle):
    c = CASES["NH3"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    for P in (ref["P"], np.random.default_rng(2).standard_normal(ref["P"].shape)):
        P = 0.5 * (P + P.T)
        assert_close(hf.formG(P, ref["int2"]), oracle.formG(P, ref["int2"]), 1e-11, 1e-11, "G")


def test_doscf_nonconvergence_is_reported(oracle):
    c = CASES["H2O"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    with pytest.raises(hf.SCFNotConverged):
        hf.doscf(ref["H"], ref["int2"], ref["S"], 5, 3, 1e-10, 1e-8, 1.0)


def test_transform_and_mbpt2_dropins(oracle):
    c = CASES["CH4_1"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    mo_ref = oracle.transform_int2(ref["int2"], ref["C"])
    mo = hf.transform_int2(ref["int2"], ref["C"])
    assert_close(mo, mo_ref, 1e-11, 1e-11, "moint2")
    e2_ref = oracle.mbpt2(mo_ref, ref["lam"], 5)
    assert abs(hf.mbpt2(mo_ref, ref["lam"], 5) - e2_ref) < 1e-12
    assert abs(e2_ref - (-0.16815509)) < 1e-7  # test_gaussians_molecules.f90:114


def test_diis_reaches_the_same_solution(oracle):
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(2, seed=11)
    o = dict(tolP=1e-10, tolE=1e-12)
    mix = hf.rhf(atno, xyz, hf.RHFOptions(nscf=100, **o))
    diis = hf.rhf(atno, xyz, hf.RHFOptions(diis=True, **o))
    assert diis["niter"] < mix["niter"]
    assert abs(mix["Etot"] - diis["Etot"]) < 1e-10
    assert abs(mix["E2"] - diis["E2"]) < 1e-9


def test_water_dimer_against_oracle(oracle):
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(2, seed=3)
    r = hf.rhf(atno, xyz, hf.RHFOptions(diis=True, tolP=1e-10, tolE=1e-12))
    ref = oracle.rhf_gauss(atno, xyz, nscf=100, tolE=1e-12, tolP=1e-10)
    e2 = oracle.mp2_semidirect(ref["int2"], ref["C"], ref["lam"], 10)
    assert abs(r["Etot"] - ref["Etot"]) < 1e-10
    assert abs(r["E2"] - e2) < 1e-8


def test_gpu_errors_are_statuses():
    from hfsolver_gb300.clusters import water

    atno, xyz = water()
    with pytest.raises(hf.SCFNotConverged):
        hf.rhf(atno, xyz, hf.RHFOptions(nscf=2))


@pytest.mark.parametrize("nw,seed", [(2, 3), (4, 0)])
def test_purification_matches_diagonalisation(nw, seed):
    """SP2 purification of the density each iteration reaches the same SCF
    solution (and the same final orbitals) as an eigensolve each iteration."""
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(nw, seed=seed)
    o = dict(diis=True, tolP=1e-10, tolE=1e-12, schwarz=1e-12)
    a = hf.rhf(atno, xyz, hf.RHFOptions(**o), want_orbitals=True)
    b = hf.rhf(atno, xyz, hf.RHFOptions(purify=True, **o), want_orbitals=True)
    assert abs(a["Etot"] - b["Etot"]) < 1e-10
    assert abs(a["E2"] - b["E2"]) < 1e-9
    assert np.max(np.abs(a["lam"] - b["lam"])) < 1e-7


def test_jk_direct_entry(oracle):
    from tests.gpu_common import basis_args

    c = CASES["NH3"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    b = ref["basis"]
    I = oracle.unpack(ref["int2"], b.n)
    P = ref["P"]
    J_ref = np.einsum("ijkl,kl->ij", I, P)
    K_ref = np.einsum("ikjl,kl->ij", I, P)
    J, K = hf.jk(*basis_args(b), P)
    assert_close(J, J_ref, 1e-11, 1e-11, "J")
    assert_close(K, K_ref, 1e-11, 1e-11, "K")
    assert_close(J - 0.5 * K, oracle.formG(P, ref["int2"]), 1e-11, 1e-11, "G")


@pytest.mark.parametrize("precision", ["fp64", "split_bf16"])
def test_mp2_energy_entry(oracle, precision):
    c = CASES["CH4_1"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    e2 = oracle.mbpt2(oracle.transform_int2(ref["int2"], ref["C"]), ref["lam"], 5)
    got = hf.mp2_energy(ref["int2"], ref["C"], ref["lam"], 5, precision)
    assert abs(got - e2) < (1e-12 if precision == "fp64" else 1e-9)


@pytest.mark.parametrize("fused", [True, False])
def test_rhf_batch_matches_single_calls(fused):
    """hfgpu_rhf_batch in both modes: molecules of one wave sharing their ERI and
    Fock-build launches (fused), or each on its own streams, give the energies
    of one-at-a-time calls."""
    from hfsolver_gb300.clusters import water, water_cluster

    mols = [water(), (np.array(CASES["CH4_1"]["atno"]), np.array(CASES["CH4_1"]["xyz"], float)),
            water_cluster(2, seed=1)]
    o = hf.RHFOptions(diis=True, tolP=1e-9, tolE=1e-11, batch_fused=fused)
    batch = hf.rhf_batch(mols, o)
    for (a, x), r in zip(mols, batch):
        single = hf.rhf(a, x, o)
        assert abs(r["niter"] - single["niter"]) <= 1
        assert abs(r["Etot"] - single["Etot"]) < 1e-11
        assert abs(r["E2"] - single["E2"]) < 1e-11


def test_fused_batch_bench_configuration_and_small_waves():
    """The batch workload's configuration (DIIS, SP2, screened incremental Fock
    builds, atomic start, tensor-core MBPT2) over uneven molecules, split into
    waves of three (batch_streams), against one-at-a-time calls."""
    from hfsolver_gb300.clusters import water_batch

    mols = water_batch(7, seed=3, nmax=4)
    o = hf.RHFOptions(nscf=60, diis=True, schwarz=1e-12, tolP=1e-10, tolE=1e-12, mp2="split_bf16", purify=True,
                      incremental=True, guess="sad", batch_streams=3)
    batch = hf.rhf_batch(mols, o)
    for (a, x), r in zip(mols, batch):
        single = hf.rhf(a, x, o)
        assert r["niter"] > 0
        assert abs(r["Etot"] - single["Etot"]) < 1e-10
        assert abs(r["E2"] - single["E2"]) < 1e-10


def test_fused_batch_molecule_failure_is_isolated():
    """A molecule that fails (an element without 6-31G** data) leaves its wave
    at once; the others finish, and the call reports the failure."""
    from hfsolver_gb300 import _lib
    from hfsolver_gb300.clusters import water, water_cluster

    mols = [water(), (np.array([8, 1, 99], dtype=np.int32), water()[1]), water_cluster(2, seed=2)]
    res = hf.rhf_batch(mols, hf.RHFOptions(diis=True))
    assert res[1]["niter"] == -_lib.ERR_INVALID
    for k in (0, 2):
        single = hf.rhf(*mols[k], hf.RHFOptions(diis=True))
        assert res[k]["niter"] > 0
        assert abs(res[k]["Etot"] - single["Etot"]) < 1e-11


def test_autotune_keeps_energies():
    """Tuned kernel shapes (timed on first use, then reused) give the same SCF
    and MBPT2 energies as the built-in rules."""
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(4, seed=2)
    o = dict(diis=True, schwarz=1e-12, tolP=1e-10, tolE=1e-12, mp2="split_bf16")
    hf.autotune_clear()
    a = hf.rhf(atno, xyz, hf.RHFOptions(**o))
    b = hf.rhf(atno, xyz, hf.RHFOptions(autotune=True, **o))
    table = hf.autotune_table()
    c = hf.rhf(atno, xyz, hf.RHFOptions(autotune=True, **o))
    assert hf.autotune_table() == table  # second molecule reuses the table
    kinds = {k for k, *_ in table}
    assert kinds == {"eri", "digest"}
    for r in (b, c):
        assert abs(r["Etot"] - a["Etot"]) < 1e-10
        assert abs(r["E2"] - a["E2"]) < 1e-9
    hf.autotune_clear()
    assert hf.autotune_table() == []


@pytest.mark.parametrize("name", [k for k in CASES if "e3" in CASES[k]])
def test_mbpt3_reference_known_answers(oracle, name):
    """mbpt3 drop-in on the reference's own H2, CH4 and H2O cases: the asserted
    E3 (test_gaussians_molecules.f90:52, :116, :191) and the oracle's terms."""
    c = CASES[name]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float), nscf=40, alpha=c["alpha"], tolE=1e-10, tolP=1e-8)
    mo = hf.transform_int2(ref["int2"], ref["C"])
    e3 = hf.mbpt3(mo, ref["lam"], c["nocc_mp2"])
    val, tol, _ = c["e3"]
    assert abs(e3 - val) < tol
    assert abs(e3 - oracle.mbpt3(mo, ref["lam"], c["nocc_mp2"])) < 1e-12


@pytest.mark.parametrize("name", [k for k in CASES if "gf" in CASES[k]])
def test_find_pole_diag_reference_known_answers(oracle, name):
    """find_pole_diag drop-in (src/gf.f90:15-34) on the reference's own H2, CH4,
    NH3, H2O and FH cases: the asserted poles (test_gaussians_molecules.f90:55,
    :119, :161, :194, :215) from the GPU's own transform_int2, and the oracle's
    pole from the same MO integrals."""
    c = CASES[name]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float), nscf=40, alpha=c["alpha"], tolE=1e-10, tolP=1e-8)
    mo = hf.transform_int2(ref["int2"], ref["C"])
    nocc = int(sum(c["atno"])) // 2
    i, val, tol, _ = c["gf"]
    Eg = hf.find_pole_diag(i, mo, ref["lam"], nocc, 200, 1e-10)
    assert abs(Eg - val) < tol, (Eg, val)
    assert abs(Eg - oracle.find_pole_diag(i, mo, ref["lam"], nocc, 200, 1e-10)) < 1e-11


def test_find_pole_diag_reports_nonconvergence(oracle):
    c = CASES["H2O"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    mo = hf.transform_int2(ref["int2"], ref["C"])
    with pytest.raises(hf.SCFNotConverged):
        hf.find_pole_diag(5, mo, ref["lam"], 5, 1, 1e-10)
