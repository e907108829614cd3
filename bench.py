#!/usr/bin/env python
"""
Benchmark: GFN2-xTB energy + forces, molecules/s, on the packed persistent
GPU path (one launch per stage for the whole batch), with p50/p99 step
latency, the per-molecule GPU path beside it, and the CPU reference.

Workload: the 256 seeded synthetic molecules of 10-60 atoms (elements
H/C/N/O/F/S) of the batched GFN2 configuration, energy AND forces (the
metric is E+F). A step is one single point (SCF + analytic gradient) of
every molecule of the batch with the inputs resident in HBM.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

N > 1 (torchrun): independent replicas, one batch per rank (weak scaling).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
# serving slots and their side streams need more hardware queues than the default 8
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "GFN2 E+F molecules/s batched vs per-molecule at |dE|<1e-8 Eh; p50/p99 ms"
WORKLOAD = "GFN2 E+F, 256 synthetic molecules of 10-60 atoms (H/C/N/O/F/S), packed batch"


def args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--count", type=int, default=256)
    p.add_argument("--cpu-sample", type=int, default=16,
                   help="molecules timed on the CPU (at the size quantiles of the set)")
    p.add_argument("--per-molecule", type=int, default=16,
                   help="molecules on the 1-by-1 GPU path (at the size quantiles of the set)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--serve-rate", type=float, default=2000.0,
                   help="Poisson arrival rate of the serving leg (0: skip the leg)")
    p.add_argument("--serve-slots", type=int, default=8)
    p.add_argument("--no-configs", action="store_true",
                   help="skip the config-1 latency and config-3 throughput legs")
    p.add_argument("--config4", action="store_true",
                   help="also run the serving configuration: 200 Poisson requests at 2000/s, "
                        "GFN1/GFN2, 8-300 atoms log-uniform, E+F, 120 GB budget")
    return p.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(index)], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip() == "Active":
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


MMA_SHAPES = {0: (8, 8, 4), 1: (16, 8, 4), 2: (16, 8, 8), 3: (16, 8, 16)}


def fp64_peaks(dev, local: int) -> dict:
    """
    Measured FP64 rates of this GPU (TFLOP/s), with the SM clock sampled
    while the probes run (about a second in total): the scalar FMA pipe
    (``dxtb_fp64_fma_probe``, the roofline denominator of the SCF) and the
    FP64 tensor-core instructions (``dxtb_fp64_mma_probe``, one entry per
    mma.sync shape).
    """
    from dxtb_gb300 import _lib

    L = _lib.lib()
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    st = _lib.stream_ptr()
    blocks, threads = sms * 8, 256

    def rate(launch, flops, reps=3):
        launch()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = 0.0
        for _ in range(reps):
            s.record()
            launch()
            e.record()
            e.synchronize()
            best = max(best, flops / (s.elapsed_time(e) * 1e-3) / 1e12)
        return best

    clocks = Clocks(local)
    t0 = time.perf_counter()
    out_d: dict = {}
    while True:
        iters = 40000
        fma = rate(lambda: _lib.check(L.dxtb_fp64_fma_probe(iters, blocks, threads, out.data_ptr(), st),
                                      "probe"), 2.0 * 8 * iters * blocks * threads)
        out_d["dfma"] = max(out_d.get("dfma", 0.0), fma)
        for sh, (m, n, k) in MMA_SHAPES.items():
            it = 4000
            r = rate(lambda: _lib.check(L.dxtb_fp64_mma_probe(sh, it, blocks, threads, out.data_ptr(), st),
                                        "probe"), 2.0 * m * n * k * 4 * it * (threads // 32) * blocks)
            key = f"dmma_m{m}n{n}k{k}"
            out_d[key] = max(out_d.get(key, 0.0), r)
        if time.perf_counter() - t0 > 1.0:
            break
    out_d["clocks"] = clocks.stop()
    return out_d


def quantile_sample(nao: np.ndarray, k: int) -> list[int]:
    """k molecules at the size quantiles of the set (sorted by orbital count,
    the middle of each of k equal slices): their mean n^3 matches the set's."""
    o = np.argsort(nao, kind="stable")
    k = min(k, len(nao))
    return [int(o[int((j + 0.5) * len(nao) / k)]) for j in range(k)]


def scf_flops(nao: np.ndarray, iters: np.ndarray, forces: bool) -> float:
    """Algorithmic FP64 work of the SCF launch (per-molecule sum): orthogonaliser
    (2/3 n^3) + 11.33 n^3 per iteration (basis transform 4n^3, tridiagonalisation
    4/3 n^3, back-transform 2n^3, C = X C' 2n^3, P = C f C^T 2n^3) + W (2 n^3)."""
    n3 = nao.astype(np.float64) ** 3
    return float(((2.0 / 3.0) + iters * (34.0 / 3.0) + (2.0 if forces else 0.0)) @ n3)


def nao_of(mols) -> np.ndarray:
    """GFN2 orbital counts of a molecule list (H 1, C/N/O/F 4, S 9)."""
    ao = {1: 1, 6: 4, 7: 4, 8: 4, 9: 4, 16: 9}
    return np.array([sum(ao[int(z)] for z in m[0]) for m in mols], dtype=np.int64)


def cpu_reference(mols, sample: int, method="gfn2"):
    """The CPU restatement of the reference path (oracle), E + F per molecule,
    on `sample` molecules at the size quantiles of the set."""
    from oracle import xtb_oracle as X

    threads = torch.get_num_threads()
    idx = quantile_sample(nao_of(mols), sample)
    sel = [mols[i] for i in idx]
    times, energies = [], []
    t0 = time.perf_counter()
    for num, pos in sel:
        t = time.perf_counter()
        r = X.singlepoint(method, num, pos, grad=True, tol=1e-10)
        times.append(time.perf_counter() - t)
        energies.append(r.energy)
    total = time.perf_counter() - t0
    return {
        "value": len(sel) / total,
        "unit": "molecules/s",
        "cores": threads,
        "kind": "port",
        "sample": (f"{len(sel)} of the {len(mols)} molecules at the size quantiles (mean n^3 "
                   f"{np.mean(nao_of(sel).astype(float) ** 3) / np.mean(nao_of(mols).astype(float) ** 3):.3f}"
                   " x the set's), sequential, E+F, float64"),
        "p50_ms": 1e3 * float(np.percentile(times, 50)),
        "p99_ms": 1e3 * float(np.percentile(times, 99)),
    }, dict(zip(idx, energies))


# the timed configuration through the public API: implicit-mode SCF with
# x_atol = f_atol = 1e-10 (energy converged to 1e-8), zero-potential start
E2E_OPTS = {"exclude": ["disp", "d4sc"], "scf_mode": "implicit", "x_atol": 1e-10, "f_atol": 1e-10,
            "maxiter": 250, "guess": "sad"}

# DRAM bytes (read + write) of the SCF launches per step: the ncu capture of
# every SCF size class on the first 16 molecules (19.33 MB for a sum of n^2 of
# 138,431, profiles/k_scf_classes_and_grad_pairs_16mol.md) scaled to the 256
# molecules by the sum of n^2 (2,392,388); the SCF's DRAM traffic is its
# O(n^2) inputs and outputs, its O(n^3) work stays in L2 and shared memory
SCF_TRAFFIC = 19.33e6 / 138431 * 2392388
SCF_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the four SCF launches, "
                      "16 molecules, scaled by sum n^2 to the 256-molecule step")


def measured_hbm_gbs() -> float | None:
    """HBM copy bandwidth of this machine's GPUs (MEASURED_PEAKS.json), if present."""
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(f.read_text())["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def set_parity(res, pb) -> dict:
    """Energies and forces of every molecule of the timed batch against the
    oracle fixture of the 256-molecule set (tests/golden/sets_c2.npz)."""
    d = np.load(ROOT / "tests" / "golden" / "sets_c2.npz")
    e = res.energy.cpu().numpy()
    g = res.gradient.cpu().numpy()
    de = np.abs(e - d["gfn2/energy"])
    df = np.array([np.abs(g[pb.atom_off[i]: pb.atom_off[i + 1]] - d["gfn2/gradient"][i, : d["nat"][i]]).max()
                   for i in range(pb.nmol)])
    return {
        "molecules": int(pb.nmol),
        "max_abs_dE": float(de.max()),
        "max_abs_dF": float(df.max()),
        "outside_tol": int(((de > 1e-8) | (df > 1e-6)).sum()),
        "tol": {"dE_Eh": 1e-8, "dF_Eh_per_bohr": 1e-6},
        "reference": "oracle float64 (tol 1e-10), all molecules of the set",
    }


def other_configs(dev, steps: int) -> dict:
    """Config 1: GFN1 E+F of C8N2O2H12 (24 atoms, n = 72) through
    GFN1Calculator, latency per call (repeated calls replay the CUDA graph),
    positions from the host. Config 3: the 64 molecules of 30-120 atoms as
    one packed batch per method, E+F, device-resident, CUDA events; every
    molecule against the oracle fixture (tests/golden/sets_c3.npz), with the
    GFN1 molecules whose oracle SCF needs over 100 iterations counted apart."""
    from dxtb_gb300 import GFN1Calculator
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run
    from dxtb_gb300.workloads import config_molecules

    out = {}
    z1, p1 = config_molecules(1)[0]
    calc = GFN1Calculator(torch.as_tensor(z1), opts={
        "scf_mode": "implicit", "x_atol": 1e-10, "f_atol": 1e-10, "maxiter": 250,
        "guess": "sad", "exclude": ["disp", "d4sc"]}, device=dev)
    hp = torch.tensor(p1).pin_memory()
    lat = []
    for k in range(3 + max(steps, 5)):
        calc.reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f = calc.get_forces(hp.to(dev, non_blocking=True)).cpu()
        e = float(calc.get_energy(hp.to(dev, non_blocking=True)))
        lat.append(time.perf_counter() - t0)
    lat = lat[3:]
    out["config1"] = {
        "workload": "GFN1 E+F, C8N2O2H12 (24 atoms, n = 72), seed 1000, through GFN1Calculator",
        "p50_ms": 1e3 * float(np.median(lat)), "min_ms": 1e3 * float(min(lat)),
        "energy": e, "cuda_graph_replay": any(g is not None for g in calc._graphs.values()),
    }
    d = np.load(ROOT / "tests" / "golden" / "sets_c3.npz")
    nat = d["nat"]
    nums = [d["numbers"][i, : nat[i]] for i in range(len(nat))]
    pos = [torch.tensor(d["positions"][i, : nat[i]]) for i in range(len(nat))]
    chaotic = {"gfn1": {1, 6, 23, 37, 48, 53}, "gfn2": set()}  # oracle > 100 iterations
    for method in ("gfn1", "gfn2"):
        pb = PackedBatch(tables(method), nums, pos, dev)
        st: dict = {}
        res = run(pb, forces=True, state=st, tol=float(d["tol"]), maxiter=int(d["maxiter"]))
        ms = []
        for _ in range(max(1, min(steps, 3))):
            s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record()
            res = run(pb, forces=True, state=st, tol=float(d["tol"]), maxiter=int(d["maxiter"]))
            e0.record()
            e0.synchronize()
            ms.append(s0.elapsed_time(e0))
        e = res.energy.cpu().numpy()
        g = res.gradient.cpu().numpy()
        de = np.abs(e - d[f"{method}/energy"])
        df = np.array([np.abs(g[pb.atom_off[i]: pb.atom_off[i + 1]] - d[f"{method}/gradient"][i, : nat[i]]).max()
                       for i in range(pb.nmol)])
        bad = (de > 1e-8) | (df > 1e-6)
        out[f"config3_{method}"] = {
            "workload": f"{method.upper()} E+F, 64 synthetic molecules of 30-120 atoms, packed batch",
            "molecules_per_s": pb.nmol / (float(np.median(ms)) * 1e-3),
            "ms_per_step": float(np.median(ms)),
            "outside_tol": int(bad.sum()),
            "outside_tol_not_chaotic": int(sum(1 for i in np.where(bad)[0] if i not in chaotic[method])),
            "chaotic_excluded": sorted(chaotic[method]),
            "max_abs_dE_others": float(max(de[i] for i in range(pb.nmol) if i not in chaotic[method])),
            "max_abs_dF_others": float(max(df[i] for i in range(pb.nmol) if i not in chaotic[method])),
        }
    return out


def main():
    a = args()
    world, rank, local = dist_setup()
    from dxtb_gb300.workloads import config_molecules

    mols = config_molecules(2, count=a.count)
    if a.impl == "reference":
        if rank != 0:
            return
        torch.set_num_threads(os.cpu_count() or 1)
        vals, lat = [], []
        cb = None
        for _ in range(a.warmup if a.warmup < 1 else 1):
            cpu_reference(mols, 1)
        for _ in range(a.steps):
            cb, _ = cpu_reference(mols, a.cpu_sample)
            vals.append(cb["value"])
        v = float(np.median(vals))
        cb["value"] = v
        line = {
            "impl": "reference", "metric": METRIC, "value": v, "unit": "molecules/s",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * a.cpu_sample / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": cb["sample"]},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "molecules/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from dxtb_gb300 import GFN2Calculator
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run

    nums = [m[0] for m in mols]
    pos = [torch.tensor(m[1]) for m in mols]
    pb = PackedBatch(tables("gfn2"), nums, pos, dev)
    state: dict = {}
    l2 = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    from dxtb_gb300 import autotune

    tuned = autotune.ensure(pb)  # size-class policy: cached, or tuned once on this batch
    for _ in range(a.warmup):
        res = run(pb, forces=True, state=state)
    torch.cuda.synchronize()
    barrier(world)
    clocks = Clocks(local)
    step_ev, stage_ev = [], []
    for k in range(a.steps):
        l2.fill_(float(k))  # flush L2 between timed steps
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        evs: dict = {}
        s.record()
        res = run(pb, forces=True, state=state, events=evs)
        e.record()
        step_ev.append((s, e))
        stage_ev.append(evs)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    step_ms = [s.elapsed_time(e) for s, e in step_ev]
    total_s = max_over_ranks(sum(step_ms) * 1e-3, world)
    stages = {
        k: float(np.mean([ev[k][0].elapsed_time(ev[k][1]) for ev in stage_ev]))
        for k in stage_ev[0]
    }
    status = res.status.cpu().numpy()
    iters = res.iterations.cpu().numpy()
    value = pb.nmol * a.steps * world / total_s

    # parity of the timed result on every molecule against the oracle fixture
    parity = set_parity(res, pb) if a.count == 256 else None

    # roofline of the dominant kernels (the persistent SCF launches)
    peaks = fp64_peaks(dev, local)
    peak = peaks["dfma"]
    flops = scf_flops(pb.nao, iters, True)
    achieved = flops / (stages["scf"] * 1e-3) / 1e12
    # integral stage: S, H0, D (3) and Q (6) written, 8 bytes each per n^2
    int_bytes = 8.0 * 11 * float((pb.nao.astype(np.float64) ** 2).sum())
    hbm_peak = measured_hbm_gbs()
    int_gbs = int_bytes / (stages["integrals"] * 1e-3) / 1e9

    # per-molecule GPU path (same kernels, one molecule per launch)
    per = []
    for i in quantile_sample(pb.nao, a.per_molecule):
        pbi = PackedBatch(tables("gfn2"), [nums[i]], [pos[i]], dev)
        sti: dict = {}
        run(pbi, forces=True, state=sti)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        run(pbi, forces=True, state=sti)
        e.record()
        e.synchronize()
        per.append(s.elapsed_time(e))
    per_mol_value = len(per) / (sum(per) * 1e-3) if per else None

    # end to end through the public API: pinned host positions in, E and F out
    e2e = None
    if not a.no_e2e:
        nmax = max(len(n) for n in nums)
        znum = torch.zeros(len(nums), nmax, dtype=torch.int64)
        hpos = torch.zeros(len(nums), nmax, 3, dtype=torch.float64).pin_memory()
        for i, (n, p) in enumerate(zip(nums, pos)):
            znum[i, : len(n)] = torch.as_tensor(n)
            hpos[i, : len(n)] = p
        calc = GFN2Calculator(znum, opts=E2E_OPTS, device=dev)
        for _ in range(a.warmup):
            dpos = hpos.to(dev, non_blocking=True)
            f = calc.get_forces(dpos)
            en = calc.get_energy(dpos)
        torch.cuda.synchronize()
        t_e2e = []
        h_e = torch.empty(len(nums), dtype=torch.float64).pin_memory()
        h_f = torch.empty_like(hpos).pin_memory()
        for k in range(a.steps):
            l2.fill_(float(k))
            calc.reset()  # no result reuse across steps: every step computes
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dpos = hpos.to(dev, non_blocking=True)
            f = calc.get_forces(dpos)
            en = calc.get_energy(dpos)
            h_f.copy_(f)
            h_e.copy_(en)
            t_e2e.append(time.perf_counter() - t0)
        e2e_s = max_over_ranks(sum(t_e2e), world)
        e2e = {
            "value": len(nums) * a.steps * world / e2e_s,
            "unit": "molecules/s",
            "h2d_bytes_per_step": int(hpos.numel() * 8),
            "d2h_bytes_per_step": int(h_f.numel() * 8 + h_e.numel() * 8),
            "p50_ms": 1e3 * float(np.percentile(t_e2e, 50)),
            "p99_ms": 1e3 * float(np.percentile(t_e2e, 99)),
            # repeated calls on the same molecules replay a captured CUDA graph
            "cuda_graph_replay": any(g is not None for g in getattr(calc, "_graphs", {}).values()),
        }

    # serving: the same molecules as a seeded Poisson request stream through the
    # continuous-batching loop; latency = arrival -> energy and forces on the host
    serving = None
    if a.serve_rate > 0:
        from dxtb_gb300.serving import CudaExecutor, Request, Server, latency_summary, warm_up

        rng = np.random.default_rng(4000)
        arr = np.cumsum(rng.exponential(1.0 / a.serve_rate, size=len(nums)))
        reqs = [Request(i, "gfn2", nums[i], mols[i][1], arrival=float(arr[i])) for i in range(len(nums))]
        ex = CudaExecutor(dev, slots=a.serve_slots)
        warm_up(ex, a.serve_slots)
        torch.cuda.synchronize()
        srv = Server(ex, hbm_budget=120e9, slots=a.serve_slots, max_pack=32, order="size")
        out = srv.serve(reqs)
        serving = latency_summary(out)
        serving.update({"rate_hz": a.serve_rate, "slots": a.serve_slots, "max_pack": 32, "order": "size",
                        "packs": srv.stats.packs, "max_inflight": srv.stats.max_inflight,
                        "hbm_budget_gb": 120.0, "status_bad": sum(1 for r in out if r.status != 0)})

    # the other single-GPU configurations: config 1 (one GFN1 molecule, E+F
    # latency through the calculator) and config 3 (64 molecules of 30-120
    # atoms, GFN1 and GFN2 E+F, packed, with parity on every molecule)
    configs = None
    if not a.no_configs and rank == 0:
        configs = other_configs(dev, a.steps)

    # the serving configuration (8-300 atoms, both methods) through the two-lane loop
    config4 = None
    if a.config4:
        from dxtb_gb300.serving import (CudaExecutor, Server, latency_summary, poisson_requests,
                                        warm_up)

        reqs = poisson_requests(200, 2000.0, 4)
        # 4 slots reserved for molecules under 160 orbitals, 8 for the rest
        # (shortest first, packs of up to 32), whose SMs are capped at 112
        # while small requests are queued or running
        slots, large_slots = 12, 8
        ex = CudaExecutor(dev, slots=slots, priorities=[-100] * (slots - large_slots) + [0] * large_slots)
        warm_up(ex, slots)
        torch.cuda.synchronize()
        srv = Server(ex, hbm_budget=120e9, slots=slots, max_pack=32, large_slots=large_slots,
                     large_n=160, large_pack=32, order="size", large_sms=112)
        c4_clocks = Clocks(local)
        out = srv.serve(reqs)
        c4_clk = c4_clocks.stop()
        config4 = latency_summary(out)
        config4["clocks"] = c4_clk
        config4.update({
            "workload": "200 requests, Poisson 2000/s (seed 4), GFN1/GFN2, 8-300 atoms log-uniform, E+F",
            "packs": srv.stats.packs, "max_inflight": srv.stats.max_inflight,
            "max_bytes_gb": srv.stats.max_bytes / 1e9, "hbm_budget_gb": 120.0,
            "iterations_max": int(max(r.iterations for r in out)),
            "status_bad": [[int(r.rid), int(r.status), int(r.iterations)] for r in out if r.status != 0],
            "slowest": sorted([[int(r.rid), round(r.latency_ms, 1), int(r.iterations)] for r in out],
                              key=lambda v: -v[1])[:5],
        })

    cpu_baseline = None
    if rank == 0 and a.cpu_sample > 0:
        cpu_baseline, ref_e = cpu_reference(mols, a.cpu_sample)
        got = res.energy.cpu().numpy()
        cpu_baseline["max_abs_dE_vs_gpu"] = float(max(abs(got[i] - e) for i, e in ref_e.items()))
    if rank != 0:
        return
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "molecules/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": float(np.mean(step_ms)),
        "p50_ms": float(np.percentile(step_ms, 50)),
        "p99_ms": float(np.percentile(step_ms, 99)),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {
            "workload": WORKLOAD,
            "molecules": pb.nmol,
            "atoms": int(pb.atom_off[-1]),
            "aos_total": int(pb.ao_off[-1]),
            "nao_min_max": [int(pb.nao.min()), int(pb.nao.max())],
            "l2": "flushed between timed steps (256 MB write)",
            "parallelism": f"replicas x{world}",
            "scf_iterations_mean_max": [float(iters.mean()), float(iters.max())],
            "status_ok": int((status == 0).sum()),
        },
        "stages_ms": stages,
        "per_molecule": {"value": per_mol_value, "unit": "molecules/s", "molecules": len(per),
                         "p50_ms": float(np.percentile(per, 50)) if per else None,
                         "p99_ms": float(np.percentile(per, 99)) if per else None},
        "speedup_vs_per_molecule": value / per_mol_value if per_mol_value else None,
        "parity": parity,
        "roofline": {
            "kernel": ("SCF launches k_scf<256,2>, k_scf<512,1>, k_scf_cluster (a CTA or a "
                       "cluster of 2-16 CTAs per molecule, by size class), over the SCF stage"),
            "bound": "fp64",
            "achieved": achieved,
            "peak": peak,
            "unit": "TFLOP/s",
            "frac": achieved / peak,
            "peak_source": "measured FP64 FMA probe (dxtb_fp64_fma_probe) on this GPU, best of the probe runs",
            "traffic": SCF_TRAFFIC,
            "traffic_source": SCF_TRAFFIC_SOURCE,
        },
        "stage_roofline": {
            "scf": {"bound": "fp64", "achieved_tflops": achieved, "frac_of_dfma": achieved / peak},
            "integrals": {"bound": "hbm", "bytes_written": int_bytes, "achieved_gbs": int_gbs,
                          "peak_gbs": hbm_peak, "frac": int_gbs / hbm_peak if hbm_peak else None},
        },
        "fp64_probes_tflops": peaks,
        "autotune": tuned,
        "cpu_baseline": cpu_baseline,
        "e2e": e2e,
        "serving": serving,
        "configs": configs,
        "config4": config4,
        "gpu_launches": res.launches * a.steps,
        "clocks": clk,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
