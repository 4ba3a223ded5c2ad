"""Analytic RHF nuclear gradients (hfgpu_rhf_gradient) against central finite
differences of the energy with h = 1e-4 bohr; tolerance 1e-6 Ha/bohr.

The single water is differenced with the oracle's energies (the reference's
own algorithm, restated on the CPU); the clusters of 2, 4, 8 and 12 waters
with the GPU energies, which agree with the oracle to 1e-12 Ha in the rest of
the suite.  Translational and rotational invariance, the torch.autograd
Function and the md.f90 minimiser close the file."""
import numpy as np
import pytest

import hfsolver_gb300 as hf
from hfsolver_gb300.clusters import water, water_cluster

pytestmark = pytest.mark.gpu

H = 1e-4
TOL = 1e-6
OPT = dict(mp2="none", diis=True, tolP=1e-11, tolE=1e-11, nscf=200)


def _fd(energy, xyz, coords):
    out = []
    for a, k in coords:
        xp = xyz.copy()
        xp[a, k] += H
        xm = xyz.copy()
        xm[a, k] -= H
        out.append((energy(xp) - energy(xm)) / (2 * H))
    return np.array(out)


def _distorted_water():
    atno, xyz = water()
    xyz = xyz.copy()
    xyz[1] += [0.05, -0.03, 0.02]
    xyz[2] += [-0.02, 0.04, -0.06]
    return atno, xyz


def test_water_gradient_vs_oracle_fd(oracle):
    atno, xyz = _distorted_water()
    _, g = hf.rhf_gradient(atno, xyz, hf.RHFOptions(**OPT))

    def e_oracle(x):
        return oracle.rhf_gauss(atno, x, nscf=200, tolE=1e-11, tolP=1e-11, diis=8)["Etot"]

    coords = [(a, k) for a in range(3) for k in range(3)]
    fd = _fd(e_oracle, xyz, coords)
    assert np.max(np.abs(g.ravel() - fd)) < TOL, (g.ravel(), fd)


def test_water_gradient_energy_matches_rhf():
    atno, xyz = _distorted_water()
    r, _ = hf.rhf_gradient(atno, xyz, hf.RHFOptions(**OPT))
    e = hf.rhf(atno, xyz, hf.RHFOptions(**OPT))["Etot"]
    assert abs(r["Etot"] - e) < 1e-11
    assert r["ms_grad"] > 0


@pytest.mark.parametrize("nw,ncoord", [(2, 18), (4, 9), (8, 12), (12, 9)])
def test_cluster_gradient_vs_fd(nw, ncoord):
    """Every coordinate of one water of the cluster (its three atoms), plus
    randomly chosen coordinates of the others up to ncoord."""
    atno, xyz = water_cluster(nw, seed=1)
    opt = hf.RHFOptions(schwarz=1e-12, **OPT)
    _, g = hf.rhf_gradient(atno, xyz, opt)
    rng = np.random.default_rng(nw)
    w = nw // 2
    coords = [(3 * w + a, k) for a in range(3) for k in range(3)]
    rest = [(a, k) for a in range(len(atno)) for k in range(3) if (a, k) not in coords]
    extra = max(0, min(ncoord, len(atno) * 3) - len(coords))
    coords += [rest[i] for i in rng.choice(len(rest), size=extra, replace=False)]

    def e_gpu(x):
        return hf.rhf(atno, x, opt)["Etot"]

    fd = _fd(e_gpu, xyz, coords)
    an = np.array([g[a, k] for a, k in coords])
    assert np.max(np.abs(an - fd)) < TOL, (coords, an, fd)


@pytest.mark.parametrize("nw", [1, 4])
def test_gradient_invariances(nw):
    atno, xyz = water_cluster(nw, seed=3) if nw > 1 else _distorted_water()
    _, g = hf.rhf_gradient(atno, xyz, hf.RHFOptions(schwarz=1e-12 if nw > 1 else 0.0, **OPT))
    # a rigid translation or rotation of the molecule leaves E unchanged
    assert np.max(np.abs(g.sum(axis=0))) < 1e-8
    torque = np.cross(xyz - xyz.mean(axis=0), g).sum(axis=0)
    assert np.max(np.abs(torque)) < 1e-7


def test_autograd_function():
    torch = pytest.importorskip("torch")
    from hfsolver_gb300.autograd import RHFEnergy

    atno, xyz = _distorted_water()
    opt = hf.RHFOptions(**OPT)
    X = torch.tensor(xyz, dtype=torch.float64, requires_grad=True)
    E = RHFEnergy.apply(X, atno, opt)
    E.backward()
    r, g = hf.rhf_gradient(atno, xyz, opt)
    assert abs(E.item() - r["Etot"]) < 1e-11
    assert np.max(np.abs(X.grad.numpy() - g)) < 1e-12
    # chain rule through a function of E
    X2 = torch.tensor(xyz, dtype=torch.float64, requires_grad=True)
    (3.0 * RHFEnergy.apply(X2, atno, opt) ** 2).backward()
    assert np.max(np.abs(X2.grad.numpy() - 6.0 * r["Etot"] * g)) < 1e-9


def test_minimize_energy_lowers_energy():
    from hfsolver_gb300 import md

    atno, xyz = _distorted_water()
    forces = md.rhf_forces(atno)
    energy = md.rhf_energy_fn(atno)
    X = xyz.T.copy()
    e0 = energy(X)
    f = md.minimize_energy(forces, energy, X, 0.02, 6)
    assert energy(X) < e0
    assert np.max(np.abs(f)) < np.max(np.abs(forces(xyz.T.copy())))
