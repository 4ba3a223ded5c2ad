"""Molecular-dynamics drivers over the analytic RHF forces.

The same integrators as hfsolver's src/md.f90, restated in numpy, with the
force callback served by hfgpu_rhf_gradient (forces = -dE/dR):
  * velocity_verlet: src/md.f90:33-56 (one step t -> t + dt, positions wrapped
    into the [0, L]^3 box);
  * minimize_energy: src/md.f90:58-86 (step along the normalised force; a step
    that lowers the energy is kept and h grows by 1.2, otherwise h shrinks by 0.2).
Arrays are (3, natoms) like the reference's X(:, j) columns.
"""
import numpy as np

from . import api


def rhf_forces(atno, options=None):
    """A forces(X) callback for the integrators: X is (3, natoms) in bohr."""
    opt = options if options is not None else api.RHFOptions(mp2="none", diis=True, tolP=1e-10, nscf=100)

    def forces(X):
        _, g = api.rhf_gradient(atno, np.asarray(X, dtype=np.float64).T, opt)
        return -g.T

    return forces


def rhf_energy_fn(atno, options=None):
    """An energy(X) callback: E_tot at positions X (3, natoms)."""
    opt = options if options is not None else api.RHFOptions(mp2="none", diis=True, tolP=1e-10, nscf=100)

    def energy(X):
        return api.rhf(atno, np.asarray(X, dtype=np.float64).T, opt)["Etot"]

    return energy


def velocity_verlet(dt, m, L, forces, f, V, X):
    """Propagates f, V, X from t to t + dt in place (src/md.f90:33-56)."""
    m3 = np.asarray(m, dtype=np.float64)[None, :]
    X += V * dt + f * dt**2 / (2 * m3)
    if np.any(np.abs(X / L) > 2):
        raise RuntimeError("X is out of range after Verlet: abs(X/L) > 2")
    X -= L * np.floor(X / L)
    f_next = forces(X)
    V += (f + f_next) * dt / (2 * m3)
    f[...] = f_next


def minimize_energy(forces, energy, X, h0, max_iter):
    """Steepest descent with an adaptive step (src/md.f90:58-86); returns the final force."""
    f = forces(X)
    h = h0
    E = energy(X)
    for _ in range(max_iter):
        fmax = np.max(np.sqrt(np.sum(f**2, axis=0)))
        if fmax == 0.0:  # at a stationary point: no direction to step in
            break
        Xnew = X + f / fmax * h
        Enew = energy(Xnew)
        if Enew < E:
            X[...] = Xnew
            E = Enew
            f = forces(X)
            h = 1.2 * h
        else:
            h = 0.2 * h
    return f
