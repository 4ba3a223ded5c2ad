"""Python mirror of hfsolver's molecular GTO interfaces over libhfgpu.

Same names and argument meaning as the reference's routines, numpy in and out:

=====================  ==============================================  =======================
this module            reference                                       libhfgpu entry point
=====================  ==============================================  =======================
getS, getT, getV       src/qc.c:6-93 (C drivers)                       hfgpu_getS/T/V
getInts                src/qc.c:95-131                                 hfgpu_getInts
getints2               src/gaussians_hfsolver.f90:13-34 (plugin)       hfgpu_getints2
doscf                  src/scf.f90:72-136                              hfgpu_doscf
formG                  src/scf.f90:26-58                               hfgpu_formG
jk                     J and K of TT, src/scf.f90:84-105               hfgpu_jk
mp2_energy             transform_int2 + mbpt2 (E2 only)                hfgpu_mp2_energy
rhf_batch              rhf_gauss over many molecules                   hfgpu_rhf_batch
transform_int2         src/mbpt.f90:11-79                              hfgpu_transform_int2
mbpt2                  src/mbpt.f90:154-159, src/mbpt2.f90:8-31        hfgpu_mbpt2
mbpt3                  src/mbpt.f90:161-169, src/mbpt3.f90:8-128       hfgpu_mbpt3
rhf_gauss / rhf        src/drivers.f90:12-51 (+ MBPT2)                 hfgpu_rhf
rhf_gradient           dE/dR for src/md.f90:13-20 (no reference)       hfgpu_rhf_gradient
=====================  ==============================================  =======================

Errors raise HFGPUError (the reference stops the process instead); an SCF
that does not converge raises SCFNotConverged, like stop_error in doscf.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import HFGPUError

_dp = _lib._dp
_ip = _lib._ip


class SCFNotConverged(HFGPUError):
    pass


def _check(code):
    if code == _lib.ERR_NOT_CONVERGED:
        raise SCFNotConverged(code, _lib.lib().hfgpu_last_error().decode())
    _lib.check(code)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def packed_size(n):
    m = n * (n + 1) // 2
    return m * (m + 1) // 2


def _basis_args(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha):
    arrs = [_i32(nprim), _i32(istart), _f64(xcenter), _f64(ycenter), _f64(zcenter), _i32(lpower), _i32(mpower),
            _i32(npower), _f64(coef), _f64(alpha)]
    n = len(arrs[0])
    for a in arrs[1:8]:
        if len(a) != n:
            raise ValueError("per-function arrays must all have length nbf")
    args = [n, _i(arrs[0]), _i(arrs[1]), _d(arrs[2]), _d(arrs[3]), _d(arrs[4]), _i(arrs[5]), _i(arrs[6]),
            _i(arrs[7]), len(arrs[8]), _d(arrs[8]), _d(arrs[9])]
    return n, args, arrs


def getS(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha):
    n, args, keep = _basis_args(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha)
    S = np.zeros((n, n), order="F")
    _check(_lib.lib().hfgpu_getS(*args, _d(S)))
    return S


def getT(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha):
    n, args, keep = _basis_args(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha)
    T = np.zeros((n, n), order="F")
    _check(_lib.lib().hfgpu_getT(*args, _d(T)))
    return T


def getV(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha, atno, x, y, z):
    n, args, keep = _basis_args(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha)
    at, xa, ya, za = _i32(atno), _f64(x), _f64(y), _f64(z)
    V = np.zeros((n, n), order="F")
    _check(_lib.lib().hfgpu_getV(*args, len(at), _i(at), _d(xa), _d(ya), _d(za), _d(V)))
    return V


def getInts(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha):
    """All unique (ij|kl) in the 8-fold packed layout (istart 0-based, as qc.c)."""
    n, args, keep = _basis_args(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha)
    out = np.zeros(packed_size(n))
    _check(_lib.lib().hfgpu_getInts(*args, _d(out)))
    return out


def getints2(nprim, istart, center, power, coef, alpha):
    """Plugin form: center(3, n), power(3, n), 1-based istart (Fortran layout)."""
    nprim, istart = _i32(nprim), _i32(istart)
    n = len(nprim)
    center = np.asfortranarray(np.asarray(center, dtype=np.float64).reshape(3, n))
    power = np.asfortranarray(np.asarray(power, dtype=np.int32).reshape(3, n))
    coef, alpha = _f64(coef), _f64(alpha)
    out = np.zeros(packed_size(n))
    _check(_lib.lib().hfgpu_getints2(n, _i(nprim), _i(istart), center.ctypes.data_as(_dp),
                                     power.ctypes.data_as(_ip), len(coef), _d(coef), _d(alpha), _d(out),
                                     len(out)))
    return out


def doscf(H, int2, S, Noccupied, Nscf, tolE, tolP, alpha):
    """Returns (C, P, lam, E0, niter); raises SCFNotConverged like stop_error."""
    H = np.asfortranarray(H, dtype=np.float64)
    S = np.asfortranarray(S, dtype=np.float64)
    int2 = _f64(int2)
    n = H.shape[0]
    if int2.size != packed_size(n):
        raise ValueError("int2 has the wrong length")
    C = np.zeros((n, n), order="F")
    P = np.zeros((n, n), order="F")
    lam = np.zeros(n)
    E0 = np.zeros(1)
    it = np.zeros(1, dtype=np.int32)
    _check(_lib.lib().hfgpu_doscf(n, H.ctypes.data_as(_dp), _d(int2), S.ctypes.data_as(_dp), int(Noccupied),
                                  int(Nscf), float(tolE), float(tolP), float(alpha), C.ctypes.data_as(_dp),
                                  P.ctypes.data_as(_dp), _d(lam), _d(E0), _i(it)))
    return C, P, lam, float(E0[0]), int(it[0])


def jk(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha, P, schwarz=0.0):
    """(J, K) of density P for a basis in the C-driver layout (integrals stay on the device)."""
    n, args, keep = _basis_args(nprim, istart, xcenter, ycenter, zcenter, lpower, mpower, npower, coef, alpha)
    P = np.asfortranarray(P, dtype=np.float64)
    J = np.zeros((n, n), order="F")
    K = np.zeros((n, n), order="F")
    _check(_lib.lib().hfgpu_jk(*args, P.ctypes.data_as(_dp), float(schwarz), J.ctypes.data_as(_dp),
                               K.ctypes.data_as(_dp)))
    return J, K


def mp2_energy(int2, C, lam, Noccupied, precision="fp64"):
    """E2 of transform_int2 + mbpt2 without the packed MO array (only (ia|jb))."""
    C = np.asfortranarray(C, dtype=np.float64)
    int2, lam = _f64(int2), _f64(lam)
    n = C.shape[0]
    if int2.size != packed_size(n):
        raise ValueError("int2 has the wrong length")
    E2 = np.zeros(1)
    prec = {"fp64": _lib.MP2_FP64, "split_bf16": _lib.MP2_SPLIT_BF16}[precision]
    _check(_lib.lib().hfgpu_mp2_energy(n, _d(int2), C.ctypes.data_as(_dp), _d(lam), int(Noccupied), prec, _d(E2)))
    return float(E2[0])


def eigh(A, B):
    """(lam, C) of A C = B C diag(lam) from the lower triangles (linalg.f90 eigh)."""
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    n = A.shape[0]
    if A.shape != (n, n) or B.shape != (n, n):
        raise ValueError("A and B must be square and of the same size")
    lam = np.zeros(n)
    C = np.zeros((n, n), order="F")
    _check(_lib.lib().hfgpu_eigh(n, A.ctypes.data_as(_dp), B.ctypes.data_as(_dp), _d(lam), C.ctypes.data_as(_dp)))
    return lam, C


def tridiag_eigen(d, e):
    """(lam, Z) of the symmetric tridiagonal matrix (diagonal d, off-diagonal e); host only."""
    d = _f64(d)
    e = _f64(e)
    n = d.size
    if n < 1 or e.size != max(n - 1, 0):
        raise ValueError("need n >= 1 diagonal and n - 1 off-diagonal elements")
    lam = np.zeros(n)
    Z = np.zeros((n, n), order="F")
    _check(_lib.lib().hfgpu_tridiag_eigen(n, _d(d), _d(e) if e.size else _d(np.zeros(1)), _d(lam),
                                          Z.ctypes.data_as(_dp)))
    return lam, Z


def boys(maxm, T):
    """F_0..F_maxm at each T, by the ERI kernels' device routine (diagnostic);
    array of shape (len(T), maxm + 1)."""
    T = _f64(np.atleast_1d(T))
    F = np.zeros((T.size, maxm + 1))
    _check(_lib.lib().hfgpu_boys(int(maxm), T.size, _d(T), F.ctypes.data_as(_dp)))
    return F


def formG(P, int2):
    """G = J - K/2 from the packed integrals (scf.f90:26-58)."""
    P = np.asfortranarray(P, dtype=np.float64)
    int2 = _f64(int2)
    n = P.shape[0]
    if int2.size != packed_size(n):
        raise ValueError("int2 has the wrong length")
    G = np.zeros((n, n), order="F")
    _check(_lib.lib().hfgpu_formG(n, P.ctypes.data_as(_dp), _d(int2), G.ctypes.data_as(_dp)))
    return G


def transform_int2(int2, C):
    C = np.asfortranarray(C, dtype=np.float64)
    int2 = _f64(int2)
    n = C.shape[0]
    out = np.zeros(packed_size(n))
    _check(_lib.lib().hfgpu_transform_int2(n, _d(int2), C.ctypes.data_as(_dp), _d(out)))
    return out


def mbpt2(moint2, lam, Noccupied):
    moint2, lam = _f64(moint2), _f64(lam)
    E2 = np.zeros(1)
    _check(_lib.lib().hfgpu_mbpt2(len(lam), _d(moint2), _d(lam), int(Noccupied), _d(E2)))
    return float(E2[0])


def mbpt3(moint2, lam, Noccupied):
    """mbpt.f90 mbpt3: the third-order energy from the packed MO integrals."""
    moint2, lam = _f64(moint2), _f64(lam)
    E3 = np.zeros(1)
    _check(_lib.lib().hfgpu_mbpt3(len(lam), _d(moint2), _d(lam), int(Noccupied), _d(E3)))
    return float(E3[0])


def find_pole_diag(i, moint2, lam, Noccupied, Nscf=200, tolE=1e-10):
    """gf.f90 find_pole_diag: the Green's-function pole of orbital i (1-based,
    as the Fortran function takes it); raises SCFNotConverged after Nscf
    iterations, where the reference stops."""
    moint2, lam = _f64(moint2), _f64(lam)
    E = np.zeros(1)
    it = np.zeros(1, dtype=np.int32)
    _check(_lib.lib().hfgpu_find_pole_diag(len(lam), _d(moint2), _d(lam), int(Noccupied), int(i), int(Nscf),
                                           float(tolE), _d(E), _i(it)))
    return float(E[0])


@dataclass
class RHFOptions:
    nscf: int = 40
    mix_alpha: float = 1.0
    tolE: float = 1e-10
    tolP: float = 1e-8
    diis: bool = False
    diis_size: int = 8
    schwarz: float = 0.0
    mp2: str = "fp64"          # "none" | "fp64" | "split_bf16"
    mp2_nocc: int = 0          # <= 0: sum(Z)/2
    purify: bool = False       # SP2 density purification instead of an eigensolve per iteration
    batch_streams: int = 0     # rhf_batch: molecules per wave (<= 0: 32), or in flight at once with batch_fused=False (<= 0: 8)
    batch_fused: bool = True   # rhf_batch: waves sharing one ERI and one Fock-build launch per quartet class
    incremental: bool = False  # Fock builds from screened density differences
    autotune: bool = False     # time candidate kernel shapes on first use, keep the fastest
    guess: str = "core"        # starting density: "core" (P = 0, the reference) | "sad" (atomic densities)
    eigensolver: str = "own"   # "own" (GPU tridiagonalisation + host tridiagonal solve) | "cusolver" (dsygvd)

    def to_c(self):
        o = _lib.Options()
        _lib.lib().hfgpu_default_options(o)
        o.nscf, o.mix_alpha, o.tolE, o.tolP = self.nscf, self.mix_alpha, self.tolE, self.tolP
        o.scf_accel = _lib.SCF_DIIS if self.diis else _lib.SCF_MIXING
        o.diis_size = self.diis_size
        o.schwarz = self.schwarz
        o.mp2 = {"none": _lib.MP2_NONE, "fp64": _lib.MP2_FP64, "split_bf16": _lib.MP2_SPLIT_BF16}[self.mp2]
        o.mp2_nocc = self.mp2_nocc
        o.purify = 1 if self.purify else 0
        o.batch_streams = self.batch_streams
        o.incremental = 1 if self.incremental else 0
        o.autotune = 1 if self.autotune else 0
        o.guess = {"core": 0, "sad": 1}[self.guess]
        o.eigensolver = {"own": 0, "cusolver": 1}[self.eigensolver]
        o.batch_mode = 0 if self.batch_fused else 1
        return o


def basis_size(atno):
    at = _i32(atno)
    return _lib.lib().hfgpu_basis_size(len(at), _i(at))


def rhf(atno, xyz, options=None, want_orbitals=False):
    """RHF (+ MBPT2) for nuclei atno at xyz (natoms x 3, bohr) in 6-31G**.

    Returns a dict with Etot, E0, Enuc, Ekin, E2, niter, nbf, nocc, the
    evaluated quartet counts and stage times; C and lam when want_orbitals."""
    opt = (options or RHFOptions()).to_c()
    at = _i32(atno)
    xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(len(at), 3))
    res = _lib.Result()
    n = basis_size(at)
    C = np.zeros((n, n), order="F") if want_orbitals and n else None
    lam = np.zeros(n) if want_orbitals and n else None
    code = _lib.lib().hfgpu_rhf(len(at), _i(at), _d(xyz), opt, res,
                                C.ctypes.data_as(_dp) if C is not None else None,
                                _d(lam) if lam is not None else None)
    _check(code)
    out = {k: getattr(res, k) for k, _ in _lib.Result._fields_ if k != "reserved"}
    if want_orbitals:
        out["C"], out["lam"] = C, lam
    return out


def rhf_gradient(atno, xyz, options=None):
    """Analytic RHF nuclear gradient dE_tot/dR (Ha/bohr, natoms x 3) at the
    converged SCF of rhf(atno, xyz, options); returns (result dict, gradient).
    Forces for the md.f90 integrators are -gradient (src/md.f90:13-20)."""
    opt = (options or RHFOptions(mp2="none")).to_c()
    at = _i32(atno)
    xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(len(at), 3))
    res = _lib.Result()
    g = np.zeros((len(at), 3))
    code = _lib.lib().hfgpu_rhf_gradient(len(at), _i(at), _d(xyz), opt, res, _d(g))
    _check(code)
    out = {k: getattr(res, k) for k, _ in _lib.Result._fields_ if k != "reserved"}
    return out, g


def autotune_table():
    """The autotuner's choices: a list of (kernel, bra type, ket type, size
    bucket, choice) tuples (see hfgpu_autotune_table)."""
    L = _lib.lib()
    n = L.hfgpu_autotune_table(None, 0)
    buf = ctypes.create_string_buffer(int(n) + 1)
    L.hfgpu_autotune_table(buf, n + 1)
    out = []
    for line in buf.value.decode().splitlines():
        k, tb, tk, b, c = line.split()
        out.append((k, int(tb), int(tk), int(b), int(c)))
    return out


def autotune_clear():
    _lib.lib().hfgpu_autotune_clear()


def rhf_batch(molecules, options=None):
    """hfgpu_rhf over a list of (atno, xyz) molecules in one call; returns a list
    of result dicts.  A molecule that failed has niter = -status and does not
    stop the others; errors of the call itself (no device, bad arguments) raise."""
    opt = (options or RHFOptions()).to_c()
    natoms = _i32([len(a) for a, _ in molecules])
    atno = _i32(np.concatenate([np.asarray(a) for a, _ in molecules]))
    xyz = _f64(np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1, 3) for _, x in molecules]).ravel())
    res = (_lib.Result * len(molecules))()
    code = _lib.lib().hfgpu_rhf_batch(len(molecules), _i(natoms), _i(atno), _d(xyz), opt, res)
    out = [{k: getattr(r, k) for k, _ in _lib.Result._fields_ if k != "reserved"} for r in res]
    if code != _lib.OK and not any(r["niter"] < 0 for r in out):
        _check(code)
    return out


def rhf_gauss(atno, xyz, Nscf=40, alpha=1.0, tolE=1e-10, tolP=1e-8):
    """drivers.f90 rhf_gauss: returns (C, lam, E0, Enuc, Ekin, Etot)."""
    r = rhf(atno, xyz, RHFOptions(nscf=Nscf, mix_alpha=alpha, tolE=tolE, tolP=tolP, mp2="none"),
            want_orbitals=True)
    return r["C"], r["lam"], r["E0"], r["Enuc"], r["Ekin"], r["Etot"]
