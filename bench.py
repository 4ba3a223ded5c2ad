#!/usr/bin/env python
"""RHF + MBPT2 throughput on GB300: molecules/s for a seeded 8-water cluster.

Workload (one step = one molecule through the whole pipeline): 8 rigid H2O
(0.9572 A, 104.52 deg) with random orientations, oxygens in an 8 A cube
(O-O >= 2.7 A, seed = rank), 6-31G** Cartesian basis (200 functions, 40
occupied); FP64 McMurchie-Davidson ERIs with a Schwarz cut of 1e-12, kept in
HBM; RHF with DIIS, SP2 density purification and incremental Fock builds
(dP < 1e-8, 4-energy window < 1e-10); AO->MO transform and MBPT2 on the tensor
cores (exact 7-bit bf16 slicing, tcgen05), with the plain FP64 transform timed
beside it on the same molecule ("mixed_vs_plain"); kernel tile shapes from the
autotuner (tuned during the warm-up steps).  Everything is rebuilt each step (the 1.6 GB
packed ERI array is larger than L2, so no L2 flush is needed between steps).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on rank 0.  `value` is molecules/s from CUDA events on the
library's stream; `e2e` repeats the measurement through the C ABI with host
buffers (coordinates in, orbitals out).  Multi-GPU: independent replicas, one
molecule per rank per step (the path has no exchange step).
`--impl reference` times hfsolver's own CPU algorithm (the oracle port of
src/cints.c THO integrals for every unique quartet, doscf's dense TT built
once, formG and dsygvd per SCF iteration, transform_int2, term1) on bounded
samples of the same workload on all host cores, scaled to one molecule, with
the serial (one-core) cost beside it.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RHF+MP2 molecules/s"
WORKLOAD = "water8_631gss_rhf_diis_schwarz1e-12_mp2"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(values):
    """Element-wise maximum of a list of floats over the ranks of the process group
    (the slowest replica sets a whole-job time); the values unchanged with one rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(rank, waters=8):
    from hfsolver_gb300.clusters import water_cluster

    # 8 waters in an 8 A cube, 16 waters in an 11 A cube; other sizes at the
    # density of the 8-water cube
    return water_cluster(waters, box=11.0 if waters == 16 else None, seed=rank)


def options(mp2="split_bf16"):
    import hfsolver_gb300 as hf

    return hf.RHFOptions(nscf=60, diis=True, diis_size=8, schwarz=1e-12, tolE=1e-10, tolP=1e-8, mp2=mp2,
                         purify=True, incremental=True, autotune=True, guess="sad")


# ---------------------------------------------------------------- CPU baseline
# The reference's SCF mixes densities linearly from P = 0; the iteration count
# used to scale its per-iteration stages is the GPU DIIS run's (14 on this
# molecule), fewer than linear mixing needs, so the CPU time is a lower bound.
REF_NITER = 14


def cpu_sample(atno, xyz, niter, ws=None, seed=0, serial=True, eri_budget_s=2.0):
    """hfsolver's per-molecule algorithm on this host's cores (oracle/refcost.py:
    THO ERIs for every unique quartet, the dense TT built once, formG and dsygvd
    per iteration, transform_int2's four loops, term1), timed on bounded
    samples and scaled to one molecule, on all host threads and, if serial, on
    one thread as the reference runs.  Returns a dict for the JSON line."""
    from oracle import oracle as O
    from oracle import refcost

    b = O.Basis(atno, xyz)
    nocc = int(sum(atno)) // 2
    if ws is None:
        ws = refcost.Workspace(b.n, nocc, seed=seed)
    rng = np.random.default_rng(seed)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    st, smp = refcost.molecule_cost(b, nocc, niter, threads, ws, rng, eri_budget_s=eri_budget_s)
    out = {"value": 1.0 / st["total"], "unit": "molecules/s", "cores": threads, "kind": "port",
           "seconds_per_molecule": st["total"],
           "stages_s": {k: round(v, 3) for k, v in st.items() if k != "total"},
           "sample": ("extrapolated from bounded samples of each stage of the reference's algorithm "
                      "(oracle/refpath.c, oracle/tho.c): " + "; ".join(f"{k}: {v}" for k, v in smp.items())
                      + f"; SCF iterations {niter}"),
           "measured_s": None}
    if serial:
        st1, smp1 = refcost.molecule_cost(b, nocc, niter, 1, ws, rng, eri_budget_s=eri_budget_s)
        out["serial"] = {"value": 1.0 / st1["total"], "unit": "molecules/s", "cores": 1,
                         "seconds_per_molecule": st1["total"],
                         "stages_s": {k: round(v, 3) for k, v in st1.items() if k != "total"}}
    out["measured_s"] = round(time.perf_counter() - t0, 2)
    return out, ws


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    atno, xyz = workload(0)
    ws = None
    per, per1, last = [], [], None
    for it in range(args.warmup + args.steps):
        timed = it >= args.warmup
        cb, ws = cpu_sample(atno, xyz, REF_NITER, ws=ws, seed=it, serial=timed, eri_budget_s=1.0)
        if timed:
            per.append(cb["seconds_per_molecule"])
            per1.append(cb["serial"]["seconds_per_molecule"])
            last = cb
    v = 1.0 / float(np.mean(per))
    cpu = dict(last)
    cpu["value"] = v
    cpu["seconds_per_molecule"] = float(np.mean(per))
    cpu["serial"]["value"] = 1.0 / float(np.mean(per1))
    cpu["serial"]["seconds_per_molecule"] = float(np.mean(per1))
    line = {"metric": METRIC, "value": v, "unit": "molecules/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(per)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "nbf": 200, "nocc": 40},
            "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": "molecules/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU run
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the roofline
# kernel for one molecule, from the ncu capture summarised under profiles/
# (keyed by roofline entry and basis size).
KERNEL_TRAFFIC = {
    ("step1", 200): {"bytes_per_molecule": 4.3775e9, "bytes_per_launch": 1.0944e9,
                     "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the 4 step-1 launches of one "
                               "8-water molecule (profiles/gather_gemm_traffic_water8.md)"},
}

def measured_peaks():
    """Peaks measured on this GPU pool (generated file), else the stated fallback."""
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return d["hbm_gbs"], d["bf16_tflops"], "measured (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, "fallback (6.8 TB/s, 1.9 PFLOP/s bf16)"


def timed_steps(L, stream, steps, fn):
    import torch

    torch.cuda.synchronize()
    n0 = L.hfgpu_kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out = [fn() for _ in range(steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out, L.hfgpu_kernel_launches() - n0


def run_gpu(args):
    import ctypes

    import torch

    import hfsolver_gb300 as hf
    from hfsolver_gb300 import _lib

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    L = _lib.lib()
    stream = torch.cuda.Stream()
    _lib.check(L.hfgpu_set_stream(ctypes.c_void_p(stream.cuda_stream)))
    atno, xyz = workload(rank, args.waters)
    main_mp2 = args.mp2
    other_mp2 = "fp64" if main_mp2 == "split_bf16" else "split_bf16"
    opt, opt_other = options(main_mp2), options(other_mp2)
    peak = ctypes.c_double(0)
    _lib.check(L.hfgpu_probe_fp64_tflops(ctypes.byref(peak)))
    hbm_peak, bf16_peak, peak_src = measured_peaks()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        hf.rhf(atno, xyz, opt)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    ms, results, launches = timed_steps(L, stream, args.steps, lambda: hf.rhf(atno, xyz, opt))
    barrier()
    clk = clocks.stop()
    # end to end through the C ABI with host buffers (coordinates in, orbitals out)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        hf.rhf(atno, xyz, opt, want_orbitals=True)
    torch.cuda.synchronize()
    ms_e2e = (time.perf_counter() - t0) * 1e3
    # the other MBPT2 precision on the same molecule, for the mixed-vs-plain comparison
    hf.rhf(atno, xyz, opt_other)
    ms_o, res_o, _ = timed_steps(L, stream, max(1, args.steps // 2), lambda: hf.rhf(atno, xyz, opt_other))
    barrier()
    if world > 1:
        ms, ms_e2e, ms_o = max_over_ranks([ms, ms_e2e, ms_o])
    if rank != 0:
        return 0
    r = results[-1]
    n = r["nbf"]
    avg = lambda k: float(np.mean([x[k] for x in results]))  # noqa: E731
    eri_ms, fock_ms, tc_ms = avg("ms_eri"), avg("ms_fock"), avg("ms_tcgemm")
    # A full Fock build digests every component quartet of the surviving shell quartets
    # once: 8 bytes read and 6 FMAs (12 flops) each, 1.5 flop/byte, above the FP64/HBM
    # balance of GB300 (1.26 TFLOP/s / 6.8 TB/s = 0.18), so the FP64 pipe bounds it.
    # Timed over the full builds only (incremental builds skip screened quartets).
    nfull = avg("n_fock_full")
    full_ms = avg("ms_fock_full") / nfull if nfull > 0 else fock_ms / r["niter"]
    elems = r["block_elems"] if r.get("block_elems") else r["n_bf_quartets"]
    roof = {
        "eri": {"kernel": "eri_class_kernel (21 classes, one ERI pass)", "bound": "fp64",
                "achieved": r["eri_flops"] / (eri_ms * 1e-3) / 1e12, "peak": peak.value, "unit": "TFLOP/s",
                "peak_source": "measured on this GPU by hfgpu_probe_fp64_tflops", "ms": eri_ms},
        "fock": {"kernel": "digest_kernel / digest_wide_kernel (21 classes, + symmetrize), one full Fock build",
                 "bound": "fp64", "achieved": 12.0 * elems / (full_ms * 1e-3) / 1e12, "peak": peak.value,
                 "unit": "TFLOP/s", "peak_source": "measured on this GPU by hfgpu_probe_fp64_tflops", "ms": fock_ms,
                 "ms_per_full_build": full_ms, "full_builds": nfull, "builds": r["niter"],
                 "hbm_GBps": 8.0 * elems / (full_ms * 1e-3) / 1e9},
    }
    o, v = r["nocc"], n - r["nocc"]
    # transform + MBPT2 work in the algorithmic unit: dense quarter transforms, no
    # permutational saving, 2 o N^4 + 2 o v N^3 + 2 o^2 v N^2 + 2 o^2 v^2 N flops;
    # the split-bf16 tensor work counted as 3x those flops (3-term split)
    dense_q = [2.0 * o * n ** 4, 2.0 * o * v * n ** 3, 2.0 * o * o * v * n ** 2, 2.0 * o * o * v * v * n]
    if r["tc_flops"] > 0:
        roof["tcgemm"] = {"kernel": "all tcgen05 sliced GEMMs of one AO->MO transform (steps 1-4)",
                          "bound": "tensor", "achieved": 3.0 * sum(dense_q) / (tc_ms * 1e-3) / 1e12,
                          "peak": bf16_peak, "unit": "TFLOP/s", "peak_source": peak_src, "ms": tc_ms,
                          "algorithmic": "3 x dense quarter-transform flops (2 o N^4 + 2 o v N^3 + 2 o^2 v N^2 "
                                         "+ 2 o^2 v^2 N)",
                          "executed_tflops": r["tc_flops"] / (tc_ms * 1e-3) / 1e12,
                          "executed": "21 bf16 products per FP64 multiply-add over the half transform"}
    s1_ms = avg("ms_tc_step1")
    if s1_ms > 0:
        nl = avg("n_tc_step1")
        executed1 = 2.0 * 21 * (n * (n + 1) / 2 * n) * o * n
        roof["step1"] = {"kernel": "sliced_gemm_gather_kernel<PackedRowsBlocked> (AO->MO step 1: packed ERIs "
                                   "gathered and sliced inside a tcgen05 GEMM)",
                         "bound": "tensor", "achieved": 3.0 * dense_q[0] / (s1_ms * 1e-3) / 1e12,
                         "peak": bf16_peak, "unit": "TFLOP/s", "peak_source": peak_src, "ms": s1_ms,
                         "launches": nl, "ms_per_launch": s1_ms / nl,
                         "algorithmic": "3 x 2 o N^4 (dense first quarter, split-bf16 counted 3x) per molecule",
                         "executed_tflops": executed1 / (s1_ms * 1e-3) / 1e12,
                         "executed": "21 bf16 products per FP64 multiply-add over the mu >= nu half"}
    for v_ in roof.values():
        v_["frac"] = v_["achieved"] / v_["peak"]
    top = "step1" if "step1" in roof else max(roof, key=lambda k: roof[k]["ms"])
    dominant = dict(roof[top])
    tr = KERNEL_TRAFFIC.get((top, n))
    dominant["traffic"] = tr["bytes_per_molecule"] if tr else None
    if tr:
        dominant["traffic_unit"] = "bytes per molecule (all launches of the kernel, as achieved)"
        dominant["traffic_per_launch"] = tr["bytes_per_launch"]
        dominant["traffic_source"] = tr["source"]
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu, _ = cpu_sample(atno, xyz, r["niter"], serial=True)
    batch = None
    if world == 1 and not args.no_batch and not args.no_cpu_baseline:
        # the batch workload beside the headline: 256 seeded clusters of 1-12 waters,
        # fused waves against the same molecules one at a time (mixed: all; plain
        # FP64: every 8th)
        from hfsolver_gb300.clusters import water_batch

        bopt = options("split_bf16")
        bopt.batch_streams = 32
        batch, _, _ = measure_batch(water_batch(256, seed=0), bopt, 1, 1, 8)
        batch["workload"] = "water_batch256_1to12_jitter0.05A_631gss_rhf_diis_schwarz1e-12_mp2, fused waves of 32"
    ro = res_o[-1]
    mixed = r if main_mp2 == "split_bf16" else ro
    plain = ro if main_mp2 == "split_bf16" else r
    line = {
        "metric": METRIC, "value": world * args.steps / (ms * 1e-3), "unit": "molecules/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD if args.waters == 8 else f"water{args.waters}_631gss_rhf_diis_schwarz1e-12_mp2",
                   "molecule": f"{args.waters} H2O, seed=rank, "
                               f"{11.0 if args.waters == 16 else 8.0 * (args.waters / 8) ** (1 / 3):.2f} A cube",
                   "nbf": n, "nocc": r["nocc"],
                   "global_batch": world, "scf": "DIIS + SP2 purification, incremental Fock builds, atomic-density start",
                   "autotune": True, "schwarz": 1e-12, "mp2": main_mp2,
                   "l2": f"no flush: each step rebuilds the {8 * (n * (n + 1) // 2) * (n * (n + 1) // 2 + 1) // 2 / 1e9:.1f} GB "
                         "packed ERI array (> 129 MB L2)",
                   "parallelism": f"replicas x{world}"},
        "results": {"Etot": r["Etot"], "E2": r["E2"], "niter": r["niter"]},
        "mixed_vs_plain": {"plain_fp64_molecules_per_s": world * len(res_o) / (ms_o * 1e-3)
                           if main_mp2 == "split_bf16" else world * args.steps / (ms * 1e-3),
                           "mixed_molecules_per_s": world * args.steps / (ms * 1e-3)
                           if main_mp2 == "split_bf16" else world * len(res_o) / (ms_o * 1e-3),
                           "dE2": abs(mixed["E2"] - plain["E2"]), "dEtot": abs(mixed["Etot"] - plain["Etot"]),
                           "mp2_ms": {"mixed": mixed["ms_mp2"], "plain_fp64": plain["ms_mp2"]}},
        "stages_ms": {"setup": avg("ms_setup"), "eri": eri_ms, "scf": avg("ms_scf"), "fock": fock_ms,
                      "mp2": avg("ms_mp2"), "tcgemm": tc_ms, "total": avg("ms_total")},
        "eri": {"quartets_per_s": r["n_bf_quartets"] / (eri_ms * 1e-3), "bf_quartets": r["n_bf_quartets"],
                "shell_quartets": r["n_quartets"], "prim_quartets": r["n_prim_quartets"],
                "md_flops": r["eri_flops"]},
        "roofline": dominant,
        "rooflines": roof,
        "e2e": {"value": world * args.steps / (ms_e2e * 1e-3), "unit": "molecules/s",
                "h2d_bytes_per_step": int(xyz.size * 8 + len(atno) * 4),
                "d2h_bytes_per_step": int((n * n + n) * 8 + ctypes.sizeof(_lib.Result))},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if batch is not None:
        line["batch"] = batch
    print(json.dumps(line))
    return 0


def measure_batch(mols, opt, steps, warmup, plain_every=4, clocks=None, barrier=None):
    """The batch workload's three throughputs on the same molecules: batched
    through hfgpu_rhf_batch (opt), all of them one at a time through the mixed
    path, every plain_every-th one at a time through plain FP64; energies
    compared with each other and with the oracle fixtures of this batch."""
    import torch

    import hfsolver_gb300 as hf

    # warm-up passes over the whole batch: the autotuner meets every (class, size)
    # it will see, so no tuning runs inside the timed region
    for _ in range(warmup):
        hf.rhf_batch(mols, opt)
    if clocks:
        clocks.start()
    if barrier:
        barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = []
    for _ in range(steps):
        res = hf.rhf_batch(mols, opt)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop() if clocks else None
    sub = list(range(0, len(mols), plain_every))
    single = options("split_bf16")
    plain = options("fp64")
    hf.rhf(mols[0][0], mols[0][1], single)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    one_mixed = [hf.rhf(a, x, single) for a, x in mols]
    torch.cuda.synchronize()
    wall_mixed = time.perf_counter() - t1
    t2 = time.perf_counter()
    one_plain = [hf.rhf(mols[i][0], mols[i][1], plain) for i in sub]
    torch.cuda.synchronize()
    wall_plain = time.perf_counter() - t2
    nbf = [r["nbf"] for r in res]
    oracle = None
    try:
        fx = json.load(open(os.path.join(ROOT, "tests", "golden", "water_clusters.json"))).get("batch")
    except (OSError, ValueError):
        fx = None
    if fx and fx["count"] == len(mols) and all(len(mols[m["index"]][0]) == 3 * m["n_waters"] for m in fx["molecules"]):
        oracle = {"molecules": [m["index"] for m in fx["molecules"]],
                  "max_dEtot": max(abs(res[m["index"]]["Etot"] - m["Etot"]) for m in fx["molecules"]),
                  "max_dE2": max(abs(res[m["index"]]["E2"] - m["E2"]) for m in fx["molecules"])}
    rec = {"molecules": len(mols), "nbf_min": min(nbf), "nbf_max": max(nbf), "nbf_mean": float(np.mean(nbf)),
           "mixed_batched_molecules_per_s": steps * len(mols) / wall,
           "mixed_one_at_a_time_molecules_per_s": len(mols) / wall_mixed,
           "plain_fp64_one_at_a_time_molecules_per_s": len(sub) / wall_plain,
           "plain_fp64_sample": f"every {plain_every}th molecule ({len(sub)}, mean "
                                f"{np.mean([nbf[i] for i in sub]):.1f} functions against {np.mean(nbf):.1f} for all)",
           "max_dE2_batched_vs_one_at_a_time_mixed": max(abs(a["E2"] - b["E2"]) for a, b in zip(res, one_mixed)),
           "vs_gpu_fp64": {"max_dE2": max(abs(res[i]["E2"] - r["E2"]) for i, r in zip(sub, one_plain)),
                           "max_dEtot": max(abs(res[i]["Etot"] - r["Etot"]) for i, r in zip(sub, one_plain))},
           "vs_oracle_fixtures": oracle,
           "failed": sum(1 for r in res if r["niter"] <= 0),
           "timing": "host wall clock between device-wide synchronizes"}
    return rec, (wall, wall_mixed, wall_plain), clk


def run_batch(args):
    """Batched molecules/s: args.batch seeded water clusters of 1-12 waters with
    Gaussian atom jitter (0.05 A) through hfgpu_rhf_batch with mixed MBPT2, in
    waves whose molecules share one ERI launch and, every SCF iteration, one
    Fock-build launch per quartet class (a replayed CUDA graph).  Beside it: the
    same molecules one at a time through the mixed path (all of them) and
    through the plain FP64 path (every 4th), and for the molecules the oracle
    fixtures hold, |dE| against the oracle."""
    import torch

    import hfsolver_gb300 as hf
    from hfsolver_gb300.clusters import water_batch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    mols = water_batch(args.batch, seed=rank)
    opt = options("split_bf16")
    opt.batch_streams = args.streams
    opt.batch_fused = not args.batch_streams_mode
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else None
    rec, walls, clk = measure_batch(mols, opt, args.steps, args.warmup, 4, ClockSampler(local), barrier)
    wall, wall_mixed, wall_plain = walls
    if world > 1:
        wall, wall_mixed, wall_plain = max_over_ranks([wall, wall_mixed, wall_plain])
    if rank != 0:
        return 0
    value = world * args.steps * len(mols) / wall
    rec["mixed_batched_molecules_per_s"] = value
    line = {
        "metric": METRIC + " (batched)", "value": value, "unit": "molecules/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"water_batch{len(mols)}_1to12_jitter0.05A_631gss_rhf_diis_schwarz1e-12_mp2",
                   "mp2": "split_bf16",
                   "batch": ("molecules of a wave share one ERI launch and one Fock-build launch per quartet class "
                             "per SCF iteration (replayed CUDA graph)" if opt.batch_fused else
                             "each molecule on its own streams"),
                   "molecules_per_wave" if opt.batch_fused else "molecules_in_flight": args.streams,
                   "autotuned_shapes": len(hf.autotune_table()),
                   "parallelism": f"replicas x{world}"},
        "batch": rec,
        "failed": rec["failed"],
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def run_grad(args):
    """Analytic RHF gradients of seeded 2/4/8/12-water clusters: ms per
    gradient call (SCF + gradient) and for the gradient kernels alone."""
    import torch

    import hfsolver_gb300 as hf
    from hfsolver_gb300.clusters import water_cluster

    torch.cuda.set_device(0)
    opt = hf.RHFOptions(nscf=100, diis=True, schwarz=1e-12, tolE=1e-10, tolP=1e-10, mp2="none")
    out = {}
    for nw in (2, 4, 8, 12):
        atno, xyz = water_cluster(nw, seed=0)
        for _ in range(args.warmup):
            hf.rhf_gradient(atno, xyz, opt)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rs = [hf.rhf_gradient(atno, xyz, opt)[0] for _ in range(args.steps)]
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) / args.steps
        out[f"water{nw}"] = {"nbf": rs[-1]["nbf"], "ms_per_call": 1e3 * wall,
                             "ms_gradient_kernels": float(np.mean([r["ms_grad"] for r in rs])),
                             "ms_gradient_eri_kernels": float(np.mean([r["ms_grad_eri"] for r in rs])),
                             "ms_energy_eri_kernels": float(np.mean([r["ms_eri"] for r in rs])),
                             "ms_scf": float(np.mean([r["ms_scf"] for r in rs])),
                             "shell_quartets": rs[-1]["n_quartets"]}
    print(json.dumps({"metric": "RHF gradient calls/s", "value": 1e3 / out["water12"]["ms_per_call"],
                      "unit": "calls/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "higher_is_better": True, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": "water12_631gss_rhf_gradient", "schwarz": 1e-12,
                                 "timing": "host wall clock between device synchronizes"},
                      "sizes": out}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mp2", default="split_bf16", choices=["fp64", "split_bf16"],
                    help="MBPT2 precision of the headline pipeline (the other one is timed beside it)")
    ap.add_argument("--waters", type=int, default=8,
                    help="cluster size (8: 200 functions, the headline workload; 16: 400 functions)")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU-baseline sample (profiling runs)")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batch-workload record of the default run (256 molecules; "
                         "--no-cpu-baseline skips it too)")
    ap.add_argument("--batch", type=int, default=0,
                    help="batched mode: this many water clusters of 1-12 waters per step")
    ap.add_argument("--streams", type=int, default=32,
                    help="batched mode: molecules per wave (or in flight at once with --batch-streams-mode)")
    ap.add_argument("--batch-streams-mode", action="store_true",
                    help="batched mode: each molecule on its own streams instead of shared launches")
    ap.add_argument("--grad", action="store_true", help="time the analytic gradient (2-12 waters)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.grad:
        return run_grad(args)
    if args.batch > 0:
        return run_batch(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
