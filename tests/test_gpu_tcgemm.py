"""The tcgen05 sliced-bf16 GEMM (hfgpu_dgemm_sliced) against an FP64 GEMM, and
the mixed-precision MBPT2 against the FP64 one.

GEMM tolerance: |C - A B| <= 2^-40 K max|A_r.| max|B_.c| per element (each
entry is kept to 2^-42 of its row's or column's power-of-two scale, which is at
most twice the row's or column's largest entry).  MBPT2: |dE2| <= 1e-8 Ha."""
import ctypes

import numpy as np
import pytest

import hfsolver_gb300 as hf

pytestmark = pytest.mark.gpu


def sliced(A, B):
    from hfsolver_gb300 import _lib

    M, K = A.shape
    N = B.shape[1]
    A = np.ascontiguousarray(A)
    Bt = np.ascontiguousarray(B.T)
    C = np.zeros((M, N))
    dp = ctypes.POINTER(ctypes.c_double)
    _lib.check(_lib.lib().hfgpu_dgemm_sliced(M, N, K, A.ctypes.data_as(dp), Bt.ctypes.data_as(dp),
                                             C.ctypes.data_as(dp)))
    return C


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 50, 200), (1000, 130, 400), (77, 321, 97)])
def test_sliced_gemm_matches_fp64(M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)) * 10.0 ** rng.uniform(-8, 3, size=(M, 1))
    A[rng.random(A.shape) < 0.1] = 0.0
    B = rng.standard_normal((K, N)) * 10.0 ** rng.uniform(-2, 2, size=(1, N))
    C = sliced(A, B)
    ref = A @ B
    bound = 2.0 ** -40 * K * np.max(np.abs(A), axis=1)[:, None] * np.max(np.abs(B), axis=0)[None, :] + 1e-300
    assert np.all(np.abs(C - ref) <= bound), float(np.max(np.abs(C - ref) / bound))


def test_sliced_gemm_exact_on_small_integers():
    rng = np.random.default_rng(3)
    A = rng.integers(-100, 100, size=(256, 192)).astype(float)
    B = rng.integers(-100, 100, size=(192, 128)).astype(float)
    assert np.array_equal(sliced(A, B), A @ B)


# 2 and 4 waters: 40 and 80 virtual orbitals (one 64- or 80-column tile); 5 and 7 waters:
# 100 and 140 (two 80-column tiles of the gather-fed steps 2 and 4, with the virtual
# slices padded to whole tiles); 1 water: 20 virtual orbitals
@pytest.mark.parametrize("nw,seed", [(1, 0), (2, 3), (4, 0), (5, 1), (7, 2)])
def test_mixed_mp2_matches_fp64(nw, seed):
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(nw, seed=seed)
    o = dict(diis=True, tolP=1e-10, tolE=1e-12)
    e64 = hf.rhf(atno, xyz, hf.RHFOptions(mp2="fp64", **o))
    emx = hf.rhf(atno, xyz, hf.RHFOptions(mp2="split_bf16", **o))
    assert abs(e64["Etot"] - emx["Etot"]) < 1e-12
    assert abs(e64["E2"] - emx["E2"]) < 1e-8


def test_sixteen_water_mixed_vs_fp64():
    """16 waters, 400 functions, 80 occupied: the tensor-core MBPT2 against the
    FP64 transform on the same SCF solution (the FP64 path itself matches the
    oracle fixtures up to 200 functions)."""
    from hfsolver_gb300.clusters import water_cluster

    atno, xyz = water_cluster(16, box=11.0, seed=0)
    o = dict(diis=True, purify=True, schwarz=1e-12, tolP=1e-8, tolE=1e-10)
    emx = hf.rhf(atno, xyz, hf.RHFOptions(mp2="split_bf16", **o))
    e64 = hf.rhf(atno, xyz, hf.RHFOptions(mp2="fp64", **o))
    assert emx["nbf"] == 400 and emx["nocc"] == 80
    assert abs(e64["Etot"] - emx["Etot"]) < 1e-10
    assert abs(e64["E2"] - emx["E2"]) < 1e-8
