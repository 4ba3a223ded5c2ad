"""ORACLE — test infrastructure only: the CPU-baseline leg of bench.py.

The cost of hfsolver's own per-molecule algorithm on this host, measured on
bounded samples and scaled to one molecule.  The stages follow the reference's
call sequence for an RHF + MBPT2 run (src/drivers.f90:12-51 and the tests'
transform_int2 + mbpt2 calls):

  ERIs       every unique (ij|kl) by THO (getInts, src/qc.c:95-131; no
             screening), timed on random unique quartets (oracle/tho.c);
  TT         the dense n^4 TT(k,l,i,j) = (ij|kl) - 1/2 (il|kj), built once
             (src/scf.f90:84-105), timed on a slab of i;
  formG      G(i,j) = sum(P * TT(:,:,i,j)) once per SCF iteration
             (src/scf.f90:26-37, :109), timed on the same slab (larger than the
             last-level cache, so its reads stream from memory like the full
             12.8 GB array's);
  eigh       LAPACK dsygvd once per iteration (src/linalg.f90:241-264), timed
             in full on a random pair of the molecule's size;
  transform  transform_int2's four quarter transforms (src/mbpt.f90:32-77),
             each timed on a sample of its outermost loop index;
  term1      the MBPT2 sum (src/mbpt2.f90:8-31) on a sample of a.

The C loops are in oracle/refpath.c.  `threads` = 1 gives the reference's
serial cost; more threads run the sampled outer loops in parallel.
"""
import time

import numpy as np

from oracle import oracle as O

_dp = O._dp
_ip = O._ip


def _bind():
    import ctypes

    L = O.lib()
    if getattr(L, "_refpath_bound", False):
        return L
    c_int, c_i64, c_dbl = ctypes.c_int, ctypes.c_int64, ctypes.c_double
    L.refpath_tt_slab.argtypes = [c_int, _dp, c_int, _ip, _dp, c_int]
    L.refpath_formG_slab.argtypes = [c_int, _dp, c_int, _dp, _dp, c_int]
    L.refpath_step1.argtypes = [c_int, _dp, _dp, c_int, _ip, _dp, c_int]
    L.refpath_step2.argtypes = [c_int, _dp, c_int, _dp, _dp, c_int]
    L.refpath_step3.argtypes = [c_int, _dp, c_int, c_i64, _dp, _dp, c_int]
    L.refpath_step4.argtypes = [c_int, _dp, c_int, _ip, _dp, _dp, c_int]
    L.refpath_term1.argtypes = [c_int, _dp, _dp, c_int, c_int, _ip, c_int]
    L.refpath_term1.restype = c_dbl
    L.refpath_set_threads.argtypes = [c_int]
    for f in ("refpath_tt_slab", "refpath_formG_slab", "refpath_step1", "refpath_step2", "refpath_step3",
              "refpath_step4", "refpath_set_threads"):
        getattr(L, f).restype = None
    L._refpath_bound = True
    return L


def _timed(f):
    t0 = time.perf_counter()
    f()
    return time.perf_counter() - t0


class Workspace:
    """Synthetic full-size operands for one basis size (the packed AO and MO
    arrays, orbitals, a density), made once and reused across samples."""

    def __init__(self, n, nocc, seed=0):
        rng = np.random.default_rng(seed)
        self.n, self.nocc = n, nocc
        size = O.n_ints(n)
        self.int2 = rng.standard_normal(size) * 1e-2
        self.moint2 = rng.standard_normal(size) * 1e-2
        C = rng.standard_normal((n, n))
        self.C = np.asfortranarray(C / np.sqrt(n))
        P = rng.standard_normal((n, n))
        self.P = np.asfortranarray(P + P.T)
        self.lam = np.sort(rng.standard_normal(n))
        self.lam[nocc:] += 2.0
        A = rng.standard_normal((n, n))
        self.F = A + A.T
        B = rng.standard_normal((n, n))
        self.S = B @ B.T / n + np.eye(n)


def molecule_cost(basis, nocc, niter, threads, ws, rng, eri_budget_s=2.0, slab=None):
    """Seconds per molecule of the reference algorithm, per stage, from bounded
    samples on `threads` host threads.  Returns (stages dict, samples dict)."""
    L = _bind()
    n = basis.n
    L.refpath_set_threads(threads)
    nq_total = O.n_ints(n)
    st, smp = {}, {}
    # ERIs: a calibration batch, then a sample sized to the budget
    q = O.random_unique_quartets(n, 200 * threads, rng)
    dt = _timed(lambda: O.eri_list(basis, q))
    nq = int(max(200 * threads, min(2e7, len(q) * eri_budget_s / max(dt, 1e-6))))
    q = O.random_unique_quartets(n, nq, rng)
    dt = _timed(lambda: O.eri_list(basis, q))
    st["eri"] = dt * nq_total / nq
    smp["eri"] = f"{nq} random unique quartets of {nq_total}, {dt:.2f} s"
    # TT slab + formG on it
    ni = slab or (4 if threads == 1 else max(16, threads))
    ni = min(ni, n)
    i_list = np.ascontiguousarray(rng.choice(n, ni, replace=False).astype(np.int32))
    TT = np.empty(ni * n * n * n)
    dt = _timed(lambda: L.refpath_tt_slab(n, O._d(ws.int2), ni, O._i(i_list), O._d(TT), threads))
    st["tt"] = dt * n / ni
    smp["tt"] = f"{ni} of {n} values of i ({TT.nbytes / 1e9:.2f} GB of TT), {dt:.2f} s"
    Gs = np.empty(ni * n)
    L.refpath_formG_slab(n, O._d(ws.P), ni, O._d(TT), O._d(Gs), threads)  # first touch
    reps = 3
    dt = _timed(lambda: [L.refpath_formG_slab(n, O._d(ws.P), ni, O._d(TT), O._d(Gs), threads)
                         for _ in range(reps)]) / reps
    st["formG"] = dt * n / ni * niter
    smp["formG"] = f"the same slab, {dt * 1e3:.1f} ms per pass, x {n / ni:.1f} x {niter} iterations"
    del TT
    # eigh (dsygvd) in full
    import scipy.linalg

    dt = _timed(lambda: scipy.linalg.eigh(ws.F, ws.S, lower=True, driver="gvd"))
    st["eigh"] = dt * niter
    smp["eigh"] = f"one dsygvd of n = {n} ({dt * 1e3:.1f} ms) x {niter}"
    # transform_int2, four steps on samples of their outer loop
    ns = max(1, min(threads, 8))
    mu = np.ascontiguousarray(rng.choice(n, ns, replace=False).astype(np.int32))
    out = np.empty(ns * n * n * n)
    t1 = _timed(lambda: L.refpath_step1(n, O._d(ws.int2), O._d(ws.C), ns, O._i(mu), O._d(out), threads))
    T_nu = out  # same shape: any contents serve for timing
    out2 = np.empty(ns * n * n * n)
    t2 = _timed(lambda: L.refpath_step2(n, O._d(ws.C), ns, O._d(T_nu), O._d(out2), threads))
    stride = 8
    ns3 = min(ns, stride)
    T2 = np.zeros(n * n * n * stride)
    t3 = _timed(lambda: L.refpath_step3(n, O._d(ws.C), ns3, stride, O._d(T2), O._d(out), threads))
    del T2
    kl = np.ascontiguousarray(rng.choice(n, ns, replace=False).astype(np.int32))
    t4 = _timed(lambda: L.refpath_step4(n, O._d(ws.C), ns, O._i(kl), O._d(out2), O._d(ws.moint2), threads))
    st["transform"] = (t1 + t2) * n / ns + t3 * n / ns3 + t4 * n / ns
    smp["transform"] = (f"{ns} of {n} outer indices per step ({t1:.2f} + {t2:.2f} + {t3:.2f} + {t4:.2f} s)")
    del out, out2
    # term1
    na = max(1, min(nocc, threads))
    al = np.ascontiguousarray(rng.choice(nocc, na, replace=False).astype(np.int32))
    dt = _timed(lambda: L.refpath_term1(n, O._d(ws.moint2), O._d(ws.lam), nocc, na, O._i(al), threads))
    st["term1"] = dt * nocc / na
    smp["term1"] = f"{na} of {nocc} values of a, {dt:.2f} s"
    st["total"] = sum(v for k, v in st.items())
    return st, smp
