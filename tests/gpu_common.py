"""Helpers shared by the GPU parity tests."""
import numpy as np


def basis_args(b):
    """Oracle basis -> per-function arrays in the reference C-driver layout."""
    return (b.nprim, b.istart, b.center[:, 0], b.center[:, 1], b.center[:, 2], b.power[:, 0], b.power[:, 1],
            b.power[:, 2], b.coef, b.alpha)


def assert_close(got, ref, atol, rtol=0.0, what=""):
    got, ref = np.asarray(got), np.asarray(ref)
    err = np.abs(got - ref)
    bound = atol + rtol * np.abs(ref)
    bad = err > bound
    assert not bad.any(), f"{what}: {bad.sum()} of {err.size} beyond tolerance, max err {err.max():.3e}"
