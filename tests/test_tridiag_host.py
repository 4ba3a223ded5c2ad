"""The host half of the eigensolver (hfgpu_tridiag_eigen): symmetric tridiagonal
eigenvalues and eigenvectors, checked against scipy's LAPACK tridiagonal solver on
the cases inverse iteration finds hard (repeated and clustered eigenvalues,
exact zeros, graded entries).  Needs no GPU."""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")


@pytest.fixture(scope="module")
def hf():
    import hfsolver_gb300 as hf

    return hf


def _check(hf, d, e, tol=1e-13):
    d, e = np.asarray(d, float), np.asarray(e, float)
    n = d.size
    lam, Z = hf.tridiag_eigen(d, e)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    ref = scipy_linalg.eigh_tridiagonal(d, e, eigvals_only=True) if n > 1 else d.copy()
    scale = max(np.abs(ref).max(), np.abs(e).max() if e.size else 0.0, 1e-300)
    assert np.all(np.diff(lam) >= 0), "eigenvalues not ascending"
    assert np.abs(lam - ref).max() <= tol * n * scale
    assert np.abs(Z.T @ Z - np.eye(n)).max() <= tol * n
    assert np.abs(T @ Z - Z * lam).max() <= tol * n * scale


@pytest.mark.parametrize("n", [1, 2, 3, 10, 200, 401])
def test_random(hf, n):
    rng = np.random.default_rng(n)
    _check(hf, rng.standard_normal(n), rng.standard_normal(n - 1))


def test_zero_and_identity(hf):
    _check(hf, np.zeros(50), np.zeros(49))
    _check(hf, np.ones(50), np.zeros(49))


def test_repeated_eigenvalues(hf):
    rng = np.random.default_rng(7)
    d = np.repeat(rng.standard_normal(20), 10)
    _check(hf, d, np.zeros(199))
    _check(hf, d, 1e-15 * rng.standard_normal(199))


def test_wilkinson_close_pairs(hf):
    m = 10
    w = np.abs(np.arange(-m, m + 1)).astype(float)
    _check(hf, w, np.ones(2 * m))
    # ten weakly coupled copies: clusters of ten nearly equal eigenvalues
    d = np.tile(w, 10)
    e = np.tile(np.r_[np.ones(2 * m), 1e-10], 10)[:-1]
    _check(hf, d, e)


def test_graded(hf):
    n = 120
    _check(hf, 10.0 ** np.linspace(-8, 2, n), 10.0 ** np.linspace(-9, 1, n - 1))


def test_invalid_input_is_a_status(hf):
    with pytest.raises(hf.HFGPUError):
        hf.tridiag_eigen(np.array([1.0, np.nan]), np.array([0.5]))


def test_concurrent_calls_share_the_pool(hf):
    """Batched molecules solve their tridiagonal problems from several host threads
    at once; the shared worker pool must give each call its own, unchanged result."""
    from concurrent.futures import ThreadPoolExecutor

    rng = np.random.default_rng(11)
    cases = [(rng.standard_normal(n), rng.standard_normal(n - 1)) for n in (150, 200, 260, 199, 64, 300)]
    serial = [hf.tridiag_eigen(d, e) for d, e in cases]
    with ThreadPoolExecutor(max_workers=6) as ex:
        for _ in range(3):
            got = list(ex.map(lambda c: hf.tridiag_eigen(*c), cases))
            for (l0, z0), (l1, z1) in zip(serial, got):
                assert np.array_equal(l0, l1)
                assert np.array_equal(z0, z1)
