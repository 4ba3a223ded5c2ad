"""Generate tests/golden/water_clusters.json with the oracle (CPU).

For seeded water clusters (hfsolver_gb300.clusters): the oracle's RHF energy
(THO integrals, DIIS to reach the same converged solution faster than linear
mixing) to dP < 1e-10, and the MBPT2 energy from the (ia|jb)-only form of
transform_int2 + term1.

* "2", "4", "8": water_cluster(n, seed=0), every unique quartet computed, as
  the reference does; also 400 packed ERIs at random positions for
  element-wise checks at full size.
* "12": water_cluster(12, seed=0) (300 functions); "16": the 16-water cluster
  of the precision workload, water_cluster(16, box=11 A, seed=0) (400
  functions).  The reference itself stops above 120 functions
  (src/basis.f90:537); here the oracle leaves out quartets whose Schwarz bound
  is below 1e-16 (the GPU path cuts at 1e-12) and sums G by one pass over the
  unique integrals.  "screen_check" records that this shortcut reproduces the
  unscreened 8-water fixture.
* "batch": a subset of the batch workload water_batch(256, seed=0) (1-12
  waters, 0.05 A Gaussian jitter): the first molecule of each of eight sizes,
  with its index in the batch, computed the same screened way.

    python tests/golden/make_fixtures.py [2 4 8 12 16 screen_check batch ...]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hfsolver_gb300.clusters import water_batch, water_cluster  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "water_clusters.json")
SCREEN = 1e-16
BATCH_SEED, BATCH_COUNT = 0, 256
# first molecule of sizes 1, 3, 5, 7, 9, 10, 11, 12 waters in water_batch(256, seed=0)
BATCH_INDICES = [5, 8, 24, 2, 15, 9, 0, 14]


def energies(atno, xyz, screen=0.0, sample_ints=0, seed_ints=0):
    t0 = time.time()
    big = screen > 0
    r = O.rhf_gauss(atno, xyz, nscf=100, tolE=1e-12, tolP=1e-10, diis=8, screen=screen, scatter=big)
    t1 = time.time()
    nocc = int(sum(atno)) // 2
    e2 = O.mp2_semidirect(r["int2"], r["C"], r["lam"], nocc)
    t2 = time.time()
    d = {"nbf": int(r["basis"].n), "nocc": nocc, "Etot": r["Etot"], "E0": r["E0"], "Enuc": r["Enuc"], "E2": e2,
         "niter_diis": r["niter"], "lam_homo": float(r["lam"][nocc - 1]),
         "seconds": {"rhf": t1 - t0, "mp2": t2 - t1}}
    if screen > 0:
        d["oracle_screen"] = screen
    if sample_ints:
        rng = np.random.default_rng(seed_ints)
        pos = np.sort(rng.choice(len(r["int2"]), size=sample_ints, replace=False))
        d["ints_pos"] = pos.tolist()
        d["ints_val"] = r["int2"][pos].tolist()
    return d


def make(nw, seed=0):
    box = 11.0 if nw == 16 else 8.0 * (nw / 8.0) ** (1 / 3)
    atno, xyz = water_cluster(nw, box=box, seed=seed)
    screen = SCREEN if nw > 8 else 0.0
    d = energies(atno, xyz, screen=screen, sample_ints=0 if nw > 8 else 400, seed_ints=1000 + nw)
    d.update({"n_waters": nw, "seed": seed, "box_ang": box})
    return d


def make_screen_check(data):
    """The screened, scatter-summed oracle against the unscreened fixture at 8 waters."""
    f = data["8"]
    atno, xyz = water_cluster(8, seed=f["seed"])
    d = energies(atno, xyz, screen=SCREEN)
    return {"n_waters": 8, "screen": SCREEN, "Etot": d["Etot"], "E2": d["E2"],
            "dEtot_vs_unscreened": d["Etot"] - f["Etot"], "dE2_vs_unscreened": d["E2"] - f["E2"],
            "seconds": d["seconds"]}


def make_batch():
    mols = water_batch(BATCH_COUNT, seed=BATCH_SEED)
    out = []
    for idx in BATCH_INDICES:
        atno, xyz = mols[idx]
        d = energies(atno, xyz, screen=SCREEN if len(atno) > 24 else 0.0)
        d.update({"index": idx, "n_waters": len(atno) // 3})
        out.append(d)
        print("batch", idx, d["nbf"], d["Etot"], d["E2"], d["seconds"], flush=True)
    return {"seed": BATCH_SEED, "count": BATCH_COUNT, "jitter_ang": 0.05, "molecules": out}


def main():
    keys = sys.argv[1:] or ["2", "4", "8"]
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for k in keys:
        if k == "screen_check":
            data[k] = make_screen_check(data)
        elif k == "batch":
            data[k] = make_batch()
        else:
            data[k] = make(int(k))
        print(k, {kk: v for kk, v in data[k].items() if kk not in ("ints_pos", "ints_val", "molecules")}, flush=True)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1)


if __name__ == "__main__":
    main()
