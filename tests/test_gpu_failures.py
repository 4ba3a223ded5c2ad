"""Device routines checked one at a time, and failure paths that return a
status instead of aborting (the reference stops the process: stop_error,
src/utils.f90:171-186).  No GPU is faulted or hung: every failure here is a
status code from the host or from a bounded device wait.

* The device Boys function of the ERI kernels (boys.cuh) against the oracle's
  Fm (src/special_functions.f90:189-248) for m <= 12 on the reference's own
  test points (src/tests/test_fm.f90:10-41) and a grid that straddles the
  switch from the Taylor table to the asymptotic form at T = 50, with
  test_fm.f90's tolerances (abs 1e-15, rel 1e-12).
* S not positive definite: the reference stops in eigh on dsygvd's info
  (src/linalg.f90:265-279); here hfgpu_eigh and the doscf drop-in return
  HFGPU_ERR_LINALG.
* The bounded grid barrier of the cooperative kernels (gridsync.cuh): a
  barrier that waits for more blocks than were launched gives up after the
  limit and reports HFGPU_ERR_CUDA; the device stays usable.
"""
import ctypes

import numpy as np
import pytest

from tests.golden_reference_answers import CASES

pytestmark = pytest.mark.gpu

XLIST = [0.0, 1e-9, 1e-6, 0.1, 0.5, 2.0, 10.0, 15.0, 19.0, 20.0, 21.0, 25.0, 30.0, 50.0, 100.0,
         150.0, 200.0, 500.0, 2000.0, 20000.0, 2e5, 2e6, 2e8]


def _rel(a, b):
    d = np.abs(a - b)
    m = np.maximum(np.abs(a), np.abs(b))
    return np.where(d < np.finfo(float).tiny, 0.0, d / np.where(m == 0, 1, m))


def test_device_boys_matches_oracle(oracle):
    import hfsolver_gb300 as hf

    # the reference's points, the Taylor grid's nodes and midpoints, and the
    # neighbourhood of the switch at T = 50
    T = np.unique(np.concatenate([
        XLIST, np.arange(0, 50, 1 / 16.0), np.arange(0, 50, 1 / 16.0) + 1 / 32.0,
        [49.9, 49.96875, 49.99, 49.999999, 50.000001, 50.01, 50.03125, 50.5, 51.0, 60.0, 102.9, 103.1],
        np.random.default_rng(3).uniform(0, 120, 400)]))
    for maxm in (0, 1, 4, 8, 12):
        F = hf.boys(maxm, T)
        for t, row in zip(T, F):
            ref = oracle.boys(maxm, float(t))
            assert np.all(np.abs(row - ref) < 1e-15), (maxm, t, row - ref)
            assert np.all(_rel(ref, row) < 1e-12), (maxm, t, _rel(ref, row))


def test_eigh_rejects_indefinite_metric():
    import hfsolver_gb300 as hf
    from hfsolver_gb300 import _lib

    rng = np.random.default_rng(5)
    n = 12
    A = rng.standard_normal((n, n))
    A = A + A.T
    B = np.eye(n)
    B[3, 3] = -0.5
    with pytest.raises(_lib.HFGPUError) as e:
        hf.eigh(A, B)
    assert e.value.code == _lib.ERR_LINALG


def test_doscf_rejects_overlap_that_is_not_positive_definite(oracle):
    """The doscf drop-in given an S with a negative direction returns
    HFGPU_ERR_LINALG in its first eigensolve, as the reference stops in eigh."""
    import hfsolver_gb300 as hf
    from hfsolver_gb300 import _lib

    c = CASES["H2O"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    S = ref["S"].copy()
    # two nearly identical functions: replace function 1 by a copy of function 0
    # rotated slightly the wrong way, which makes S indefinite
    S[1, :] = S[0, :]
    S[:, 1] = S[:, 0]
    S[1, 1] = S[0, 0] - 1e-3
    with pytest.raises(_lib.HFGPUError) as e:
        hf.doscf(ref["H"], ref["int2"], S, 5, 40, 1e-10, 1e-8, 1.0)
    assert e.value.code == _lib.ERR_LINALG
    # the library is still usable
    C, P, lam, E0, it = hf.doscf(ref["H"], ref["int2"], ref["S"], 5, 40, 1e-10, 1e-8, 1.0)
    assert abs(E0 - ref["E0"]) < 1e-10


def test_grid_barrier_completes_and_times_out():
    from hfsolver_gb300 import _lib

    L = _lib.lib()
    ms = ctypes.c_double(0)
    assert L.hfgpu_grid_barrier_check(8, 8, 1000.0, ctypes.byref(ms)) == _lib.OK, L.hfgpu_last_error()
    assert ms.value < 1000.0
    # one block arrives at a barrier that waits for two: the wait runs out
    rc = L.hfgpu_grid_barrier_check(1, 2, 20.0, ctypes.byref(ms))
    assert rc == _lib.ERR_CUDA
    assert b"timed out" in L.hfgpu_last_error()
    assert 19.0 <= ms.value < 1000.0, ms.value
    # every block of a wider grid gives up too, and the device stays usable
    rc = L.hfgpu_grid_barrier_check(16, 64, 10.0, ctypes.byref(ms))
    assert rc == _lib.ERR_CUDA
    assert L.hfgpu_grid_barrier_check(4, 4, 1000.0, ctypes.byref(ms)) == _lib.OK, L.hfgpu_last_error()
    import hfsolver_gb300 as hf
    from hfsolver_gb300.clusters import water

    r = hf.rhf(*water(), hf.RHFOptions(mp2="none"))
    assert np.isfinite(r["Etot"])
