"""Generate tests/golden/water_clusters.json with the oracle (CPU, minutes).

For seeded water clusters (hfsolver_gb300.clusters.water_cluster) of 2, 4 and
8 waters: the oracle's RHF energy (THO integrals for every unique quartet, no
screening, as the reference computes them; DIIS to reach the same converged
solution faster than linear mixing) to dP < 1e-10, and the MBPT2 energy from
the (ia|jb)-only form of transform_int2 + term1.  Also a few hundred packed
ERIs at random positions, for element-wise checks at full size.

    python tests/golden/make_fixtures.py [n_waters ...]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hfsolver_gb300.clusters import water_cluster  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "water_clusters.json")


def make(nw, seed=0):
    atno, xyz = water_cluster(nw, seed=seed)
    t0 = time.time()
    r = O.rhf_gauss(atno, xyz, nscf=100, tolE=1e-12, tolP=1e-10, diis=8)
    t1 = time.time()
    nocc = int(sum(atno)) // 2
    e2 = O.mp2_semidirect(r["int2"], r["C"], r["lam"], nocc)
    t2 = time.time()
    rng = np.random.default_rng(1000 + nw)
    pos = np.sort(rng.choice(len(r["int2"]), size=400, replace=False))
    return {"n_waters": nw, "seed": seed, "box_ang": 8.0 * (nw / 8.0) ** (1 / 3), "nbf": int(r["basis"].n),
            "nocc": nocc, "Etot": r["Etot"], "E0": r["E0"], "Enuc": r["Enuc"], "E2": e2,
            "niter_diis": r["niter"], "lam_homo": float(r["lam"][nocc - 1]),
            "ints_pos": pos.tolist(), "ints_val": r["int2"][pos].tolist(),
            "seconds": {"rhf": t1 - t0, "mp2": t2 - t1}}


def main():
    sizes = [int(a) for a in sys.argv[1:]] or [2, 4, 8]
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for nw in sizes:
        d = make(nw)
        data[str(nw)] = d
        print(nw, d["nbf"], d["Etot"], d["E2"], d["seconds"], flush=True)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1)


if __name__ == "__main__":
    main()
