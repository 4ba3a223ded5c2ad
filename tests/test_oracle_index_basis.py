"""Oracle packed index and basis layout against src/tests/test_ijkl.f90:20-45
and src/tests/test_basis.f90:1-58."""
import numpy as np
import pytest


@pytest.mark.parametrize("n", [1, 2, 10, 50])
def test_ijkl_enumeration(oracle, n):
    # enumerate (i,j,k,l), i>=j, k>=l, ij>=kl in the reference's loop order
    quads = []
    for i in range(n):
        for j in range(i + 1):
            ij = i * (i + 1) // 2 + j
            for k in range(n):
                for l in range(k + 1):
                    if ij >= k * (k + 1) // 2 + l:
                        quads.append((i, j, k, l))
    q = np.array(quads, dtype=np.int64)
    expect = np.arange(len(q))
    i, j, k, l = q.T
    for perm in [(i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k), (k, l, i, j), (l, k, i, j),
                 (k, l, j, i), (l, k, j, i)]:
        assert np.array_equal(oracle.ijkl(*perm), expect)
    assert len(q) == n * (n ** 3 + 2 * n ** 2 + 3 * n + 2) // 8
    # the C index agrees with the vectorised one
    lib = oracle.lib()
    for t in range(0, len(q), max(1, len(q) // 50)):
        assert lib.oracle_ijkl(*[int(x) for x in q[t]]) == t


def test_cartesian_shell_order(oracle):
    assert oracle.cartesian_shell(0) == [(0, 0, 0)]
    assert [p[0] for p in oracle.cartesian_shell(1)] == [1, 0, 0]
    s2 = oracle.cartesian_shell(2)
    assert [p[0] for p in s2] == [2, 1, 1, 0, 0, 0]
    assert [p[1] for p in s2] == [0, 1, 0, 2, 1, 0]
    assert [p[2] for p in s2] == [0, 0, 1, 0, 1, 2]
    s3 = oracle.cartesian_shell(3)
    assert [p[0] for p in s3] == [3, 2, 2, 1, 1, 1, 0, 0, 0, 0]
    assert [p[1] for p in s3] == [0, 1, 0, 2, 1, 0, 3, 2, 1, 0]
    assert [p[2] for p in s3] == [0, 0, 1, 0, 1, 2, 0, 1, 2, 3]
    s4 = oracle.cartesian_shell(4)
    assert [p[0] for p in s4] == [4, 3, 3, 2, 2, 2, 1, 1, 1, 1, 0, 0, 0, 0, 0]
    assert [p[1] for p in s4] == [0, 1, 0, 2, 1, 0, 3, 2, 1, 0, 4, 3, 2, 1, 0]
    assert [p[2] for p in s4] == [0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 0, 1, 2, 3, 4]


def test_getstart_and_sizes(oracle):
    assert oracle.getstart([6, 3, 3, 1, 1, 1]) == [1, 7, 10, 13, 14, 15]
    assert oracle.getstart([6, 6, 6, 3, 3, 1, 1, 1]) == [1, 7, 13, 19, 22, 25, 26, 27]
    m = 15 * 16 // 2
    assert oracle.n_ints(15) == m * (m + 1) // 2


def test_water_basis_size(oracle):
    b = oracle.Basis([8, 1, 1], [[0, 0, 0], [1.809, 0, 0], [-0.453549, 1.751221, 0]])
    assert b.n == 25  # O: s6 s3 p3 s1 p1 d1 = 15, each H: s3 s1 p1 = 5


def test_unknown_element_rejected(oracle):
    with pytest.raises(ValueError):
        oracle.Basis([99], [[0, 0, 0]])
