#!/usr/bin/env python
"""Benchmark of the two-site DMRG hot path on GB300.

Workload: spinful Fermi-Hubbard open chain, L=32, t=1, U=4, mu=0, local dim 4,
(N, 2Sz) = (32, 0), max bond dimension 256, 5 Lanczos iterations, SVD
truncation 1e-10, seeded random initial MPS (seed 42, the reference's
generator). A step is one full two-site sweep (left-to-right and
right-to-left). Inputs are synthetic (built by the package's Hamiltonian
builder and seeded MPS generator).

Arms:
  default             libctgpu.so (CUDA kernels for sm_103a) through dmrg_twosite.
  --impl reference    the reference's CPU algorithm (the C restatement in oracle/,
                      bit-identical to the reference where both build) on all host cores.

Output: one JSON line on rank 0. Timing rules: W warm-up sweeps, then K timed
sweeps; each sweep starts on an idle device after a 256 MiB buffer (> L2) has
been overwritten; device time from CUDA events on the library's stream around
each sweep; max over ranks. Multi-GPU runs are independent replicas (a DMRG
sweep is sequential over bonds; nothing is exchanged).
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

WORKLOAD = {"workload": "fermi_hubbard_1d L=32 t=1 U=4 mu=0 (N,2Sz)=(32,0) D=256 maxiter=5 tol=1e-10 seed=42",
            "nsites": 32, "t": 1.0, "u": 4.0, "mu": 0.0, "max_vdim": 256, "maxiter_lanczos": 5,
            "tol_split": 1e-10, "rng_seed": 42}
METRIC = "two-site DMRG sweeps/s (Fermi-Hubbard L=32, D=256)"
UNIT = "sweeps/s"
L2_FLUSH_BYTES = 256 << 20
PRECISIONS = {"fp64": 0, "bf16x3": 1}


def build_inputs():
    from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native
    w = WORKLOAD
    H = hm.fermi_hubbard_1d(w["nsites"], w["t"], w["u"], w["mu"])
    sector = hm.encode_quantum_number_pair(w["nsites"], 0)
    c = native.random_mps(w["nsites"], 4, hm.HUBBARD_QSITE, sector, w["max_vdim"], w["rng_seed"])
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    return H, psi0


def chain_bytes(ch) -> int:
    n = 0
    for t in ch.tensors:
        n += 8 * t.num_elements_blocks() + 8 * 2 * t.ndim + 4 * sum(len(q) for q in t.qnums_logical)
    return n


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)
            self.f.close()

    def summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_oracle_sweeps(H, psi0, sweeps: int, threads: int):
    """The reference algorithm on the host cores: per-sweep wall times and energies."""
    import oracle
    from chemtensor_gb300 import ctstructs as cs
    port = oracle.port()
    used = port.oracle_set_num_threads(threads)
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en = np.zeros(sweeps)
    ent = np.zeros(H.nsites - 1)
    w = WORKLOAD
    ret = port.oracle_dmrg_twosite(C.byref(cH), sweeps, w["maxiter_lanczos"], w["tol_split"], w["max_vdim"],
                                   C.byref(cP), en.ctypes.data, ent.ctypes.data)
    times = np.zeros(sweeps)
    n = port.oracle_get_sweep_times(times.ctypes.data, sweeps)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    if ret != 0:
        raise RuntimeError(f"oracle dmrg failed: {ret}")
    return times[:n], en, used


def bench_reference(args, world, rank):
    if rank != 0:
        return
    H, psi0 = build_inputs()
    threads = os.cpu_count() or 1
    times, en, used = run_oracle_sweeps(H, psi0, args.warmup + args.steps, threads)
    t = float(np.sum(times[args.warmup:]))
    value = args.steps / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD["workload"], "l2": "not applicable (host CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": used, "kind": "port",
                         "sample": f"sweeps {args.warmup}..{args.warmup + args.steps - 1} of one dmrg_twosite call "
                                   f"(C restatement of the reference, OpenMP over blocks, OpenBLAS)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "energy_last_sweep": float(en[-1]),
    }
    print(json.dumps(line), flush=True)


def bench_gpu(args, world, rank, local):
    from chemtensor_gb300 import ctstructs as cs, native
    lib = native.lib()
    lib.ctgpu_set_device(local)
    native.set_precision(PRECISIONS[args.precision])
    H, psi0 = build_inputs()
    w = WORKLOAD
    K, W = args.steps, args.warmup
    cH = cs.make_c_mpo(H)

    def call(sweeps: int):
        cP = cs.make_c_mps(psi0)
        en = np.zeros(sweeps)
        ent = np.zeros(H.nsites - 1)
        t0 = time.perf_counter()
        ret = lib.dmrg_twosite(C.byref(cH), sweeps, w["maxiter_lanczos"], w["tol_split"], w["max_vdim"],
                               C.byref(cP), en.ctypes.data, ent.ctypes.data)
        wall = time.perf_counter() - t0
        if ret != 0:
            raise RuntimeError(f"dmrg_twosite failed: {ret} {native.last_error()}")
        out = cs.read_mps(cP)
        cs.free_mps(cP)
        return wall, en, out

    # 1) device-resident timing: W warm-up sweeps then K timed sweeps in one call
    lib.ctgpu_set_l2_flush_bytes(L2_FLUSH_BYTES)
    lib.ctgpu_set_profiling(0, 0)
    barrier(world)
    with ClockSampler(local) as clk:
        _, en, _ = call(W + K)
    sweep_ms, sweep_launches = native.sweep_times()
    t_dev = float(np.sum(sweep_ms[W:W + K])) / 1e3
    t_dev = dist_max(t_dev, world)
    value = world * K / t_dev
    launches = int(np.sum(sweep_launches[W:W + K]))

    # 2) roofline pass: same workload with every launch timed by kernel class
    lib.ctgpu_set_profiling(1, W)
    call(W + K)
    lib.ctgpu_set_profiling(0, 0)
    prof = native.kernel_profile()
    stats = native.last_stats()
    g = prof["block_gemm"]
    fp64_peak = float(lib.ctgpu_measure_fp64_tflops())
    achieved = (g["flops"] / (g["ms"] * 1e-3)) / 1e12 if g["ms"] > 0 else 0.0
    total_prof_ms = sum(v["ms"] for v in prof.values())
    roofline = {
        "bound": "fp64", "kernel": "k_gemm_f64 (grouped block GEMM, all local-H and environment contractions)",
        "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak if fp64_peak > 0 else None,
        "peak_source": "FP64 FMA probe measured live in this run (no FP64 entry in MEASURED_PEAKS.json)",
        "traffic": None, "launches": g["launches"], "flops_per_launch": g["flops"] / max(g["launches"], 1),
        "avg_launch_us": 1e3 * g["ms"] / max(g["launches"], 1),
        "kernel_share": {k: (v["ms"] / total_prof_ms if total_prof_ms > 0 else 0) for k, v in prof.items()},
    }

    # 3) end to end through the C ABI with host buffers (upload, setup, K sweeps, download)
    lib.ctgpu_set_l2_flush_bytes(0)
    barrier(world)
    wall, en_e2e, out = call(K)
    wall = dist_max(wall, world)
    e2e = {"value": world * K / wall, "unit": UNIT,
           "h2d_bytes_per_step": (chain_bytes(H) + chain_bytes(psi0)) / K,
           "d2h_bytes_per_step": chain_bytes(out) / K,
           "note": "whole dmrg_twosite call from host structs: upload, right-normalisation, environments, "
                   "K sweeps, download; per step = per sweep"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * t_dev / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "bf16x3": "bf16x3+f32acc, final sweep f64"}[args.precision],
        "data": "synthetic",
        "config": {"workload": w["workload"], "precision": args.precision, "parallelism": f"replicas x{world}",
                   "l2": "256 MiB buffer overwritten before every sweep"},
        "clocks": clk.summary(), "gpu_launches": launches, "roofline": roofline, "e2e": e2e,
        "energy_last_sweep": float(en[-1]),
        "breakdown_ms_per_sweep": {"lanczos": stats["lanczos_ms"] / max(stats["sweeps"], 1),
                                   "svd_split": stats["split_ms"] / max(stats["sweeps"], 1),
                                   "svd_max_jacobi_sweeps": stats["svd_max_sweeps"],
                                   "host_planning": 1e3 * stats["host_plan_s"] / max(stats["sweeps"], 1),
                                   "plan_cache_hit_rate": stats["plan_hits"] / max(stats["plan_hits"] + stats["plan_misses"], 1)},
        # device time of each kernel class per profiled sweep (CUDA events around every launch;
        # the difference to ms_per_step is time the device waits for the host)
        "kernel_ms_per_sweep": {k: v["ms"] / K for k, v in prof.items()},
    }

    # 4) CPU baseline on rank 0: the reference algorithm on the host cores, one sweep
    if rank == 0 and not args.no_cpu_baseline:
        times, en_cpu, used = run_oracle_sweeps(H, psi0, 1, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": 1.0 / float(times[0]), "unit": UNIT, "cores": used, "kind": "port",
                                "sample": "first sweep of the same workload from the same start state "
                                          "(C restatement of the reference; OpenMP over blocks, OpenBLAS)",
                                "energy_after_sweep": float(en_cpu[0])}
    if rank == 0:
        print(json.dumps(line), flush=True)
    cs.free_mpo(cH)


def sweeps_only(args, local):
    """One dmrg_twosite call of warmup + steps sweeps on the workload (profiler target)."""
    from chemtensor_gb300 import ctstructs as cs, native
    lib = native.lib()
    lib.ctgpu_set_device(local)
    native.set_precision(PRECISIONS[args.precision])
    H, psi0 = build_inputs()
    w = WORKLOAD
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    n = args.warmup + args.steps
    en, ent = np.zeros(n), np.zeros(H.nsites - 1)
    ret = lib.dmrg_twosite(C.byref(cH), n, w["maxiter_lanczos"], w["tol_split"], w["max_vdim"], C.byref(cP),
                           en.ctypes.data, ent.ctypes.data)
    ms, la = native.sweep_times()
    print(f"ret {ret} energies {en.tolist()} sweep_ms {ms.tolist()} launches {la.tolist()}", flush=True)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    if ret != 0:
        raise SystemExit(1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=sorted(PRECISIONS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="full", choices=["full", "sweeps"],
                    help="sweeps: only one device call of warmup+steps sweeps (for profiler captures), no JSON line")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.mode == "sweeps":
        sweeps_only(args, local)
        return
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")
    if args.impl == "reference":
        bench_reference(args, world, rank)
    else:
        bench_gpu(args, world, rank, local)
    barrier(world)


if __name__ == "__main__":
    main()
