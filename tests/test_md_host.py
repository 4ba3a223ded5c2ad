"""Host-side checks of the md.f90 integrators restated in hfsolver_gb300.md,
with analytic model forces (no GPU)."""
import numpy as np

from hfsolver_gb300 import md


def test_velocity_verlet_harmonic_oscillator():
    # one particle in a harmonic well, k = m = 1: x(t) = cos t
    k, m, L, dt = 1.0, np.array([1.0]), 1000.0, 1e-3
    centre = np.array([[500.0], [500.0], [500.0]])
    X = centre + np.array([[1.0], [0.0], [0.0]])
    V = np.zeros((3, 1))

    def forces(Y):
        return -k * (Y - centre)

    f = forces(X)
    steps = 1000
    for _ in range(steps):
        md.velocity_verlet(dt, m, L, forces, f, V, X)
    t = steps * dt
    assert abs(X[0, 0] - 500.0 - np.cos(t)) < 1e-6
    assert abs(V[0, 0] + np.sin(t)) < 1e-6
    energy = 0.5 * V[0, 0] ** 2 + 0.5 * (X[0, 0] - 500.0) ** 2
    assert abs(energy - 0.5) < 1e-6


def test_velocity_verlet_wraps_into_box():
    L = 10.0
    X = np.array([[9.9], [0.05], [5.0]])
    V = np.array([[1.0], [-1.0], [0.0]])
    f = np.zeros((3, 1))
    md.velocity_verlet(0.2, np.array([1.0]), L, lambda Y: np.zeros_like(Y), f, V, X)
    assert np.allclose(X[:, 0], [0.1, 9.85, 5.0])


def test_minimize_energy_quadratic():
    A = np.diag([1.0, 2.0, 3.0])
    x0 = np.array([[1.0], [2.0], [3.0]])

    def energy(Y):
        d = (Y - x0)[:, 0]
        return 0.5 * d @ A @ d

    def forces(Y):
        return -(A @ (Y - x0))

    X = np.zeros((3, 1))
    f = md.minimize_energy(forces, energy, X, 0.1, 300)
    assert energy(X) < 1e-6
    assert np.max(np.abs(f)) < 2e-3
