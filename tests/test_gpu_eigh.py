"""The generalized eigensolver (hfgpu_eigh: GPU Householder tridiagonalisation in
one cooperative kernel + host tridiagonal solve + compact-WY back-transform)
against scipy's LAPACK dsygvd-equivalent, and the SCF with it against the SCF
with cuSOLVER dsygvd.  Tolerances: eigenvalues 1e-12 of the spectral norm,
B-orthonormality 1e-12, residual A C - B C diag(lam) 1e-11 of the norm."""
import numpy as np
import pytest

import hfsolver_gb300 as hf

pytestmark = pytest.mark.gpu
scipy_linalg = pytest.importorskip("scipy.linalg")


def _spd(rng, n):
    M = rng.standard_normal((n, n))
    return M @ M.T / n + np.eye(n)


def _check(A, B, lam, C, tol=1e-12):
    n = A.shape[0]
    ref = scipy_linalg.eigh(A, B, eigvals_only=True)
    scale = np.abs(ref).max()
    assert np.abs(lam - ref).max() <= tol * scale * max(1, n / 50)
    assert np.abs(C.T @ B @ C - np.eye(n)).max() <= tol * max(1, n / 50)
    assert np.abs(A @ C - B @ C * lam).max() <= 10 * tol * scale * max(1, n / 50)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 17, 64, 200, 333, 512])
def test_random_pairs(n):
    rng = np.random.default_rng(100 + n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    B = _spd(rng, n)
    lam, C = hf.eigh(A, B)
    _check(A, B, lam, C)


def test_only_lower_triangles_are_read():
    rng = np.random.default_rng(5)
    n = 150
    A = rng.standard_normal((n, n))
    A = A + A.T
    B = _spd(rng, n)
    lam, C = hf.eigh(A, B)
    junk = np.triu(rng.standard_normal((n, n)), 1)
    lam2, C2 = hf.eigh(np.tril(A) + junk, np.tril(B) + junk)
    assert np.array_equal(lam, lam2)
    assert np.array_equal(C, C2)


def test_degenerate_spectra():
    rng = np.random.default_rng(9)
    n = 120
    B = _spd(rng, n)
    # A = B: every eigenvalue is 1, any B-orthonormal basis is an answer
    lam, C = hf.eigh(B, B)
    _check(B, B, lam, C)
    # eigenvalues repeated three times (like the t2 orbitals of methane)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    w = np.repeat(rng.standard_normal(n // 3), 3)
    A = Q @ np.diag(w) @ Q.T
    A = 0.5 * (A + A.T)
    lam, C = hf.eigh(A, np.eye(n))
    _check(A, np.eye(n), lam, C)
    # already diagonal (every Householder column is zero) and already tridiagonal
    D = np.diag(rng.standard_normal(n))
    lam, C = hf.eigh(D, np.eye(n))
    _check(D, np.eye(n), lam, C)
    T = np.diag(rng.standard_normal(n)) + np.diag(np.ones(n - 1), 1) + np.diag(np.ones(n - 1), -1)
    lam, C = hf.eigh(T, B)
    _check(T, B, lam, C)


def test_fock_matrix_of_a_water_cluster():
    """S and F of 8 waters (200 functions): the SCF's own problem."""
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(4, seed=2)
    r = hf.rhf(atno, xyz, hf.RHFOptions(diis=True, tolP=1e-10, tolE=1e-12, mp2="none"), want_orbitals=True)
    lam, C = r["lam"], r["C"]
    n = lam.size
    assert np.all(np.diff(lam) >= 0)
    # the same call with cuSOLVER's dsygvd
    r2 = hf.rhf(atno, xyz, hf.RHFOptions(diis=True, tolP=1e-10, tolE=1e-12, mp2="none", eigensolver="cusolver"),
                want_orbitals=True)
    assert abs(r["Etot"] - r2["Etot"]) < 1e-10
    assert r["niter"] == r2["niter"]
    assert np.abs(lam - r2["lam"]).max() < 1e-9
    # occupied-space projectors agree (orbital signs and rotations inside degenerate sets may not)
    o = r["nocc"]
    P1 = C[:, :o] @ C[:, :o].T
    P2 = r2["C"][:, :o] @ r2["C"][:, :o].T
    assert np.abs(P1 - P2).max() < 1e-8
    assert n == r["nbf"]


@pytest.mark.parametrize("solver", ["own", "cusolver"])
def test_purified_scf_and_mp2_with_either_eigensolver(solver):
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(3, seed=4)
    base = dict(diis=True, tolP=1e-10, tolE=1e-12, mp2="fp64")
    ref = hf.rhf(atno, xyz, hf.RHFOptions(**base))
    r = hf.rhf(atno, xyz, hf.RHFOptions(purify=True, eigensolver=solver, **base))
    assert abs(r["Etot"] - ref["Etot"]) < 1e-10
    assert abs(r["E2"] - ref["E2"]) < 1e-9
