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
import tempfile
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
PRECISIONS = {"fp64": 0, "bf16x3": 1, "tf32": 2, "bf16x6": 3}
# dram__bytes_read.sum + dram__bytes_write.sum of one k_svd_tour launch (ncu, see profiles/)
SVD_TRAFFIC_PER_LAUNCH = 496384


def build_inputs(host_only: bool = False):
    """The workload's MPO and seeded start state. host_only: the start state comes from the oracle's
    generator (bit-identical to the package's, which lives in the GPU library), so that the CPU arm
    loads no GPU library at all."""
    from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm
    w = WORKLOAD
    H = hm.fermi_hubbard_1d(w["nsites"], w["t"], w["u"], w["mu"])
    sector = hm.encode_quantum_number_pair(w["nsites"], 0)
    if host_only:
        import oracle
        q = np.ascontiguousarray(hm.HUBBARD_QSITE, dtype=np.int32)
        c = cs.MPS()
        if oracle.port().oracle_construct_random_mps(w["nsites"], 4, q.ctypes.data, sector, w["max_vdim"],
                                                     w["rng_seed"], C.byref(c)) != 0:
            raise RuntimeError("oracle_construct_random_mps failed")
    else:
        from chemtensor_gb300 import native
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
        out_dir = os.environ.get("CTGPU_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"ctgpu_clocks_{os.getpid()}_dev{device}.csv")

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
    local_world = int(os.environ.get("LOCAL_WORLD_SIZE", str(world)))
    if local_world > 1:
        # replicas share the host: split its cores among the ranks' lowering threads
        os.environ.setdefault("CTGPU_HOST_THREADS", str(max(1, (os.cpu_count() or 1) // local_world)))
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
    return run_oracle_sweeps_for(H, psi0, sweeps, threads, WORKLOAD["max_vdim"])


def run_oracle_sweeps_for(H, psi0, sweeps: int, threads: int, max_vdim: int):
    import oracle
    from chemtensor_gb300 import ctstructs as cs
    port = oracle.port()
    used = port.oracle_set_num_threads(threads)
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en = np.zeros(sweeps)
    ent = np.zeros(H.nsites - 1)
    w = WORKLOAD
    ret = port.oracle_dmrg_twosite(C.byref(cH), sweeps, w["maxiter_lanczos"], w["tol_split"], max_vdim,
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
    H, psi0 = build_inputs(host_only=True)
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

    # 1) device-resident timing: W warm-up sweeps then K timed sweeps in one call (first call of the
    # process: the work lists of each sweep are built as its block structures appear)
    lib.ctgpu_clear_plan_cache()
    lib.ctgpu_set_l2_flush_bytes(L2_FLUSH_BYTES)
    lib.ctgpu_set_profiling(0, 0)
    barrier(world)
    with ClockSampler(local) as clk:
        _, en, _ = call(W + K)
    sweep_ms, sweep_launches = native.sweep_times()
    timed_stats = native.last_stats()
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
    fp64_peak = float(lib.ctgpu_measure_fp64_tflops())
    total_prof_ms = sum(v["ms"] for v in prof.values())
    nsw = max(stats["sweeps"], 1)
    # dominant kernel class: the block SVD, bound by the FP64 pipe (no tensor-core or HBM bound applies:
    # its columns live in shared memory and L2)
    sv = prof["block_svd"]
    svd_flops_per_sweep = stats["svd_flops"] / nsw
    svd_ms_per_sweep = sv["ms"] / K if K > 0 else 0.0
    svd_launches_per_sweep = sv["launches"] / K if K > 0 else 0.0
    achieved = (svd_flops_per_sweep / (svd_ms_per_sweep * 1e-3)) / 1e12 if svd_ms_per_sweep > 0 else 0.0
    g = prof["block_gemm"]
    g_achieved = (g["flops"] / (g["ms"] * 1e-3)) / 1e12 if g["ms"] > 0 else 0.0
    roofline = {
        "bound": "fp64", "kernel": "k_svd_tour (block SVD: pivoted QR + cluster Jacobi, one launch per cluster size)",
        "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak if fp64_peak > 0 else None,
        "peak_source": "FP64 FMA probe measured live in this run (MEASURED_PEAKS.json has HBM and bf16 peaks only)",
        "flops_definition": "FP64 Jacobi inner products and rotations as executed and the FP32-to-FP64 "
                            "hand-over (counted on the device), QR and output factors at full rank (host "
                            "estimate); the FP32 preconditioning sweeps are not counted",
        "flops_per_launch": svd_flops_per_sweep / max(svd_launches_per_sweep, 1e-9),
        "avg_launch_us": 1e3 * svd_ms_per_sweep / max(svd_launches_per_sweep, 1e-9),
        "traffic": SVD_TRAFFIC_PER_LAUNCH,
        "traffic_source": "dram read+write of one k_svd_tour launch (the 41st of the run: one cluster-size group "
                          "of a bond, 56 CTAs) from profiles/k_svd_tour_hubbard_L32_D256.md",
        "kernel_share": {k: (v["ms"] / total_prof_ms if total_prof_ms > 0 else 0) for k, v in prof.items()},
        "block_gemm": {"bound": "fp64", "achieved": g_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                       "frac": g_achieved / fp64_peak if fp64_peak > 0 else None, "launches": g["launches"],
                       "flops_per_launch": g["flops"] / max(g["launches"], 1),
                       "avg_launch_us": 1e3 * g["ms"] / max(g["launches"], 1)},
    }

    # 3) end to end through the C ABI with host buffers (upload, setup, K sweeps, download), starting
    # from an empty plan cache like a first call
    lib.ctgpu_set_l2_flush_bytes(0)
    lib.ctgpu_clear_plan_cache()
    barrier(world)
    wall, en_e2e, out = call(K)
    wall = dist_max(wall, world)
    e2e = {"value": world * K / wall, "unit": UNIT,
           "h2d_bytes_per_step": (chain_bytes(H) + chain_bytes(psi0)) / K,
           "d2h_bytes_per_step": chain_bytes(out) / K,
           "note": "whole dmrg_twosite call from host structs with an empty plan cache: upload, "
                   "right-normalisation, environments, K sweeps from the start state, download; per step = per sweep"}

    # 4) the same workload in mixed precision: split-BF16 local-H GEMMs on the tensor cores in every
    # sweep but the last, which is FP64 (so the returned state and energies are FP64 results); same
    # timing discipline as (1)
    native.set_precision(PRECISIONS["bf16x3"])
    lib.ctgpu_clear_plan_cache()
    lib.ctgpu_set_l2_flush_bytes(L2_FLUSH_BYTES)
    barrier(world)
    _, en_mx, _ = call(W + K)
    ms_mx, _ = native.sweep_times()
    st_mx = native.last_stats()
    native.set_precision(PRECISIONS["fp64"])
    lib.ctgpu_set_l2_flush_bytes(0)
    bulk = ms_mx[W:W + K - 1] if K > 1 else ms_mx[W:W + K]
    t_bulk = dist_max(float(np.sum(bulk)) / 1e3, world)
    t_all = dist_max(float(np.sum(ms_mx[W:W + K])) / 1e3, world)
    mixed = {"precision": "bf16x3 (split-BF16, 3 products, FP32 accumulate) in sweeps 0..W+K-2, FP64 in the last",
             "sweeps_per_s_reduced": world * len(bulk) / t_bulk if t_bulk > 0 else None,
             "sweeps_per_s_incl_final_fp64": world * K / t_all if t_all > 0 else None,
             "speedup_reduced_vs_fp64": (world * len(bulk) / t_bulk) / value if t_bulk > 0 else None,
             "energy_last_sweep": float(en_mx[-1]),
             "abs_dE_vs_fp64_arm": abs(float(en_mx[-1]) - float(en[-1])),
             "max_abs_dE_over_sweeps": float(np.max(np.abs(en_mx - en))),
             "lanczos_ms_per_sweep": st_mx["lanczos_ms"] / max(st_mx["sweeps"], 1),
             "split_ms_per_sweep": st_mx["split_ms"] / max(st_mx["sweeps"], 1)}

    # 5) local-Hamiltonian microbenchmark (synthetic D = 1024, 41 Gaussian sectors, Dw = 26)
    local_h = local_h_measure(lib, args.matvecs)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * t_dev / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else f"{args.precision}+f32acc, final sweep f64",
        "data": "synthetic",
        "config": {"workload": w["workload"], "precision": args.precision, "parallelism": f"replicas x{world}",
                   "l2": "256 MiB buffer overwritten before every sweep"},
        "clocks": clk.summary(), "gpu_launches": launches, "roofline": roofline, "e2e": e2e,
        "energy_last_sweep": float(en[-1]),
        "mixed_precision": mixed, "local_h": local_h, "tile_tuning": native.tile_tuning(),
        "breakdown_ms_per_sweep": {"lanczos": stats["lanczos_ms"] / max(stats["sweeps"], 1),
                                   "svd_split": stats["split_ms"] / max(stats["sweeps"], 1),
                                   "svd_max_jacobi_sweeps": stats["svd_max_sweeps"],
                                   "host_planning": 1e3 * stats["host_plan_s"] / max(stats["sweeps"], 1),
                                   "plan_cache_hit_rate": stats["plan_hits"] / max(stats["plan_hits"] + stats["plan_misses"], 1)},
        # device time of each kernel class per profiled sweep (CUDA events around every launch;
        # the difference to ms_per_step is time the device waits for the host)
        "kernel_ms_per_sweep": {k: v["ms"] / K for k, v in prof.items()},
        # the timed call itself (first call of the process): its own plan-cache traffic and host planning
        "timed_call": {"plan_cache_hit_rate": timed_stats["plan_hits"] /
                       max(timed_stats["plan_hits"] + timed_stats["plan_misses"], 1),
                       "host_planning_ms_per_sweep": 1e3 * timed_stats["host_plan_s"] / max(timed_stats["sweeps"], 1),
                       "env_ms_per_sweep": timed_stats["env_ms"] / max(timed_stats["sweeps"], 1),
                       "lanczos_ms_per_sweep": timed_stats["lanczos_ms"] / max(timed_stats["sweeps"], 1),
                       "split_ms_per_sweep": timed_stats["split_ms"] / max(timed_stats["sweeps"], 1)},
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


LOCAL_H_PRECISIONS = (("fp64", 0, 1), ("bf16x3", 1, 3), ("tf32", 2, 1), ("bf16x6", 3, 6))   # name, ctgpu_set_precision value, products issued


def local_h_measure(lib, matvecs: int) -> dict:
    """Local-Hamiltonian microbenchmark: synthetic a, h2, l, r (D = 1024 over 41 Gaussian sectors,
    sigma = 6 sectors, Dw = 26, seeded N(0,1) blocks), operands resident, work lists built once,
    `matvecs` back-to-back applications per precision timed with CUDA events. Returns per precision
    ms per application and algorithmic TFLOP/s, the relative Frobenius error of each reduced precision
    against FP64, and the tensor-core fraction against MEASURED_PEAKS.json."""
    from chemtensor_gb300 import ctstructs as cs, native, workloads as wl
    a, h2, l, r = wl.local_h_microbench(D=1024, nsec=41, sigma=6.0, Dw=26, seed=1)
    ca, ch, cl, cr = (cs.BlockSparseTensor() for _ in range(4))
    for t, c in ((a, ca), (h2, ch), (l, cl), (r, cr)):
        cs.write_bst(t, c)
    out, results = {}, {}
    old_prec = native.set_precision(0)
    try:
        for name, prec, _ in LOCAL_H_PRECISIONS:
            native.set_precision(prec)
            ms, fl = C.c_double(), C.c_double()
            n = matvecs if prec != 0 else max(1, matvecs // 5)
            ret = lib.ctgpu_time_local_hamiltonian(C.byref(ca), C.byref(ch), C.byref(cl), C.byref(cr), n,
                                                   C.byref(ms), C.byref(fl))
            if ret != 0:
                raise RuntimeError(native.last_error())
            b = cs.BlockSparseTensor()
            if lib.ctgpu_apply_local_hamiltonian(C.byref(ca), C.byref(ch), C.byref(cl), C.byref(cr), C.byref(b)) != 0:
                raise RuntimeError(native.last_error())
            results[name] = cs.read_bst(b)
            cs.free_bst(b)
            per = ms.value / n
            out[name] = {"ms_per_matvec": per, "tflops": fl.value / (per * 1e-3) / 1e12, "flops_per_matvec": fl.value,
                         "matvecs_timed": n}
    finally:
        native.set_precision(old_prec)
        for c in (ca, ch, cl, cr):
            cs.free_bst(c)
    den = sum(float(np.sum(v ** 2)) for v in results["fp64"].blocks.values())
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    for name, prec, products in LOCAL_H_PRECISIONS:
        if prec == 0:
            continue
        num = sum(float(np.sum((results[name].blocks[k] - v) ** 2)) for k, v in results["fp64"].blocks.items())
        out[name]["rel_error_vs_fp64"] = (num / den) ** 0.5 if den > 0 else None
        out[name]["products_issued"] = products
        if "bf16_tflops" in peaks:
            out[name]["tensor_frac_issued"] = products * out[name]["tflops"] / peaks["bf16_tflops"]
            out[name]["tensor_frac_algorithmic"] = out[name]["tflops"] / peaks["bf16_tflops"]
    out["workload"] = "local_h_microbench D=1024 nsec=41 sigma=6 Dw=26 d=4 seed=1 (operands resident)"
    out["peak_source"] = "MEASURED_PEAKS.json bf16_tflops (burst)" if "bf16_tflops" in peaks else None
    return out


def bench_local_h(args, world, rank, local):
    """Local-Hamiltonian microbenchmark as its own JSON line (see local_h_measure)."""
    from chemtensor_gb300 import native
    lib = native.lib()
    lib.ctgpu_set_device(local)
    out = local_h_measure(lib, args.matvecs)
    fp64_peak = float(lib.ctgpu_measure_fp64_tflops())
    line = {
        "metric": "local-H TFLOP/s (synthetic D=1024, 41 Gaussian sectors, Dw=26)", "value": out["bf16x3"]["tflops"],
        "unit": "TFLOP/s", "n_gpus": 1, "steps": args.matvecs, "warmup": 3,
        "ms_per_step": out["bf16x3"]["ms_per_matvec"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16x3+f32acc", "data": "synthetic (seeded N(0,1) blocks)",
        "config": {"workload": "local_h_microbench D=1024 nsec=41 sigma=6 Dw=26 d=4 seed=1", "l2": "operands resident"},
        "local_h": out,
        "roofline": {"bound": "tensor", "achieved": out["bf16x3"]["tflops"], "peak": None, "unit": "TFLOP/s",
                     "note": "algorithmic FLOPs (2 m n k of the FP64 product); the split-BF16 form issues 3x that "
                             "on the tensor cores", "fp64_peak_live": fp64_peak,
                     "fp64_frac": out["fp64"]["tflops"] / fp64_peak if fp64_peak > 0 else None},
    }
    if "tensor_frac_issued" in out["bf16x3"]:
        line["roofline"]["peak"] = out["bf16x3"]["tflops"] / out["bf16x3"]["tensor_frac_algorithmic"]
        line["roofline"]["frac"] = out["bf16x3"]["tensor_frac_issued"]
        line["roofline"]["peak_source"] = "MEASURED_PEAKS.json bf16_tflops (burst); frac counts the 3 products"
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_serve(args, world, rank, local):
    """Serving mix: a seeded Poisson stream of Heisenberg / Hubbard ground-state solves (L 8..48,
    D 16..256, 2 sweeps each), replayed once by one solver thread (serial plain-FP64 solves, the
    baseline) and once by --workers solver threads sharing the GPU in the arithmetic of
    --serve-precision, with inputs built ahead by a producer thread."""
    from chemtensor_gb300 import native, serving
    lib = native.lib()
    lib.ctgpu_set_device(local)
    reqs = serving.generate_requests(args.requests, args.rate, seed=2024)
    prec = PRECISIONS[args.serve_precision]
    # warm-up: the first solves pay for context creation, kernel loading and (reduced precision) the
    # autotuner's first timings
    for p in sorted({0, prec}):
        serving.SolverPool(workers=1, device=local, sweeps=1, precision=p).run(serving.generate_requests(6, 0.0, seed=7))
    serial_pool = serving.SolverPool(workers=1, device=local)
    serial = serving.summarize(serial_pool.run(reqs))
    pool = serving.SolverPool(workers=args.workers, device=local, precision=prec, prefetch=2 * args.workers)
    conc = serving.summarize(pool.run(reqs))
    energies = {r.rid: r.energy for r in pool.results}
    ref = {r.rid: r.energy for r in serial_pool.results}
    de = [abs(energies[k] - ref[k]) for k in ref if np.isfinite(energies.get(k, np.nan)) and np.isfinite(ref[k])]
    line = {
        "metric": "DMRG serving throughput (Heisenberg/Hubbard mix, L 8-48, D 16-256, 2 sweeps)",
        "value": conc["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": args.requests, "warmup": 3,
        "ms_per_step": 1e3 / conc["solves_per_s"] if conc["solves_per_s"] else None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == 0 else f"{args.serve_precision}+f32acc (products chosen by the autotuner), final sweep f64",
        "data": "synthetic (seeded request stream)",
        "config": {"workload": f"{args.requests} requests, Poisson rate {args.rate}/s, seed 2024", "workers": args.workers,
                   "precision": args.serve_precision, "prefetch": 2 * args.workers},
        "concurrent": conc, "serial_fp64": serial,
        "speedup_vs_serial": (conc["solves_per_s"] / serial["solves_per_s"]) if serial["solves_per_s"] else None,
        "max_abs_dE_vs_serial_fp64": max(de) if de else None,
        "energy_checksum": float(sum(energies.values())),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_molecular(args, world, rank, local):
    """Molecular workload: spin-orbital Hamiltonian of n spatial orbitals with the synthetic integrals
    of workloads.molecular_integrals (seed 7), (N, 2Sz) = (n, 0), bond dimension D, seeded random
    start state (seed 42), 5 Lanczos iterations, tol 1e-10. The same start state is run once in
    plain FP64 and once in split-BF16 with the final sweep in FP64; both report device time per
    sweep (CUDA events) and the energies, and the line gives the speed-up and |dE| between them."""
    from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native, workloads as wl
    lib = native.lib()
    lib.ctgpu_set_device(local)
    n, D, S = args.orbitals, args.mol_vdim, args.mol_sweeps
    tk, vi = wl.molecular_integrals(n, seed=7)
    t0 = time.perf_counter()
    H = hm.spin_molecular(tk, vi)
    t_mpo = time.perf_counter() - t0
    c = native.random_mps(n, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(n, 0), D, 42)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    cH = cs.make_c_mpo(H)
    runs = {}
    for spec in args.mol_precisions.split(","):
        # "bf16x3env": split-BF16 also in the environment updates of the reduced-precision sweeps;
        # a suffix ":k" runs the last k sweeps in FP64 (default 1)
        name, _, fin = spec.partition(":")
        lib.ctgpu_set_final_fp64_sweeps(int(fin) if fin else 1)
        if fin:
            name = spec
        native.set_precision(PRECISIONS[name.split(":")[0].replace("env", "")])
        lib.ctgpu_set_reduced_environments(1 if name.split(":")[0].endswith("env") else 0)
        lib.ctgpu_clear_plan_cache()
        lib.ctgpu_set_profiling(1 if args.mol_profile else 0, 0)
        cP = cs.make_c_mps(psi0)
        en, ent = np.zeros(S), np.zeros(n - 1)
        t0 = time.perf_counter()
        with ClockSampler(local) as clk:
            ret = lib.dmrg_twosite(C.byref(cH), S, 5, 1e-10, D, C.byref(cP), en.ctypes.data, ent.ctypes.data)
        wall = time.perf_counter() - t0
        if ret != 0:
            raise RuntimeError(f"dmrg_twosite failed: {ret} {native.last_error()}")
        ms, la = native.sweep_times()
        st = native.last_stats()
        runs[name] = {"sweep_ms": [float(x) for x in ms], "energies": en.tolist(), "wall_s": wall,
                      "max_bond_dim": st["max_bond_dim"], "matvec_tflops": st["matvec_flops"] / max(st["lanczos_ms"], 1e-9) / 1e9,
                      "lanczos_ms_per_sweep": st["lanczos_ms"] / S, "split_ms_per_sweep": st["split_ms"] / S,
                      "env_ms_per_sweep": st["env_ms"] / S, "host_plan_s": st["host_plan_s"], "clocks": clk.summary()}
        if args.mol_profile:
            runs[name]["kernel_ms_per_sweep"] = {k: v["ms"] / S for k, v in native.kernel_profile().items()}
        cs.free_mps(cP)
        lib.ctgpu_set_profiling(0, 0)
    native.set_precision(0)
    lib.ctgpu_set_reduced_environments(0)
    lib.ctgpu_set_final_fp64_sweeps(1)
    cs.free_mpo(cH)
    oracle_leg = None
    if args.mol_oracle_sweeps > 0 and rank == 0:
        # the reference algorithm (the C restatement, bit-identical to the reference where both build)
        # from the same start state on all host cores: the FP64 anchor of the |dE| figures
        times, en_o, used = run_oracle_sweeps_for(H, psi0, args.mol_oracle_sweeps, os.cpu_count() or 1, D)
        oracle_leg = {"sweeps": args.mol_oracle_sweeps, "energies": en_o.tolist(), "s_per_sweep": times.tolist(),
                      "cores": used, "kind": "port"}
        for name, r in runs.items():
            k = min(len(r["energies"]), args.mol_oracle_sweeps)
            r["abs_dE_vs_oracle_per_sweep"] = [abs(r["energies"][i] - en_o[i]) for i in range(k)]
    line = {"metric": f"two-site DMRG sweep time (spin-orbital molecular Hamiltonian n={n}, D={D})",
            "unit": "ms/sweep", "higher_is_better": False, "n_gpus": 1, "steps": S, "warmup": 0,
            "data": "synthetic (seeded integrals and start state)",
            "config": {"workload": f"spin molecular n={n} (N,2Sz)=({n},0) D={D} maxiter=5 tol=1e-10 "
                                   f"integrals seed=7 start seed=42", "mpo_bond_dims_max": max(
                                       t.dim_logical[0] for t in H.tensors), "mpo_build_s": t_mpo},
            "runs": runs, "oracle": oracle_leg}
    mixed = [k for k in runs if k != "fp64"]
    if "fp64" in runs and mixed:
        a = runs["fp64"]
        # a reduced-precision run's last sweep is FP64: compare the mean of the bulk sweeps after the first
        bulk = lambda r, k: float(np.mean(r["sweep_ms"][1:k])) if k > 1 else float(r["sweep_ms"][0])
        for name in mixed:
            b = runs[name]
            b["speedup_bulk_sweeps_vs_fp64"] = bulk(a, S - 1) / bulk(b, S - 1)
            b["speedup_total_vs_fp64"] = sum(a["sweep_ms"]) / sum(b["sweep_ms"])
            b["abs_dE_final_vs_fp64"] = abs(a["energies"][-1] - b["energies"][-1])
        line["mixed_run"] = mixed[0]
        line["value"] = bulk(runs[mixed[0]], S - 1)
        line["speedup_total_vs_fp64"] = runs[mixed[0]]["speedup_total_vs_fp64"]
        line["abs_dE_final"] = runs[mixed[0]]["abs_dE_final_vs_fp64"]
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_singlesite(args, world, rank, local):
    """Single-site DMRG (dmrg_singlesite) on the two-site workload's Hamiltonian (Fermi-Hubbard L=32,
    U=4) from a seeded start state of bond dimension D=256 (bond dimensions stay fixed): W warm-up
    sweeps then K timed sweeps in one call, device time per sweep from CUDA events; the C
    restatement of the reference times one sweep on the host cores beside it."""
    from chemtensor_gb300 import ctstructs as cs, native
    lib = native.lib()
    lib.ctgpu_set_device(local)
    native.set_precision(0)
    H, psi0 = build_inputs()
    K, W = args.steps, args.warmup
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en = np.zeros(W + K)
    lib.ctgpu_clear_plan_cache()
    with ClockSampler(local) as clk:
        ret = lib.dmrg_singlesite(C.byref(cH), W + K, WORKLOAD["maxiter_lanczos"], C.byref(cP), en.ctypes.data)
    if ret != 0:
        raise RuntimeError(f"dmrg_singlesite failed: {ret} {native.last_error()}")
    ms, la = native.sweep_times()
    t_dev = float(np.sum(ms[W:W + K])) / 1e3
    t_dev = dist_max(t_dev, world)
    # <psi|psi> of the result on the device (ctgpu_mps_vdot)
    nrm = C.c_double()
    t0 = time.perf_counter()
    lib.ctgpu_mps_norm(C.byref(cP), C.byref(nrm))
    t_norm = time.perf_counter() - t0
    cs.free_mps(cP)
    cs.free_mpo(cH)
    line = {"metric": "single-site DMRG sweeps/s (Fermi-Hubbard L=32, D=256)", "value": world * K / t_dev,
            "unit": "sweeps/s", "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": 1e3 * t_dev / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD["workload"].replace("D=256", "D=256 (fixed)") + " dmrg_singlesite",
                       "parallelism": f"replicas x{world}"},
            "clocks": clk.summary(), "gpu_launches": int(np.sum(la[W:W + K])),
            "energies": en.tolist(), "norm_after": nrm.value, "mps_norm_wall_ms": 1e3 * t_norm}
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        port = oracle.port()
        cH2, cP2 = cs.make_c_mpo(H), cs.make_c_mps(psi0)
        e2 = np.zeros(1)
        used = port.oracle_set_num_threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        port.oracle_dmrg_singlesite(C.byref(cH2), 1, WORKLOAD["maxiter_lanczos"], C.byref(cP2), e2.ctypes.data)
        dt = time.perf_counter() - t0
        cs.free_mps(cP2)
        cs.free_mpo(cH2)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "sweeps/s", "cores": used, "kind": "port",
                                "sample": "first sweep from the same start state (C restatement of the reference)",
                                "energy_after_sweep": float(e2[0]), "gpu_energy_after_sweep": float(en[0])}
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_complex(args, world, rank, local):
    """complex128 two-site DMRG: the Fermi-Hubbard MPO (L=16, U=4) with random phases on its virtual
    bonds (the same operator) and a start state of bond dimension 64 with a random phase on every
    entry; W warm-up sweeps then K timed sweeps in one call, device time per sweep from CUDA events.
    The host baseline is the C restatement on the real form of the same problem (it has no complex
    path), one sweep."""
    from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native, workloads as wl
    lib = native.lib()
    lib.ctgpu_set_device(local)
    native.set_precision(0)
    L, D = 16, 64
    Hr = hm.fermi_hubbard_1d(L, 1.0, 4.0, 0.0)
    c = native.random_mps(L, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(L, 0), D, 42)
    psir = cs.read_mps(c)
    cs.free_mps(c)
    H = wl.complex_gauge(Hr, 5)
    psi0 = wl.complex_gauge(psir, 6, entry_phases=True)
    K, W = args.steps, args.warmup
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en, ent = np.zeros(W + K), np.zeros(L - 1)
    lib.ctgpu_clear_plan_cache()
    with ClockSampler(local) as clk:
        ret = lib.dmrg_twosite(C.byref(cH), W + K, 5, 1e-10, D, C.byref(cP), en.ctypes.data, ent.ctypes.data)
    if ret != 0:
        raise RuntimeError(f"dmrg_twosite failed: {ret} {native.last_error()}")
    ms, la = native.sweep_times()
    t_dev = dist_max(float(np.sum(ms[W:W + K])) / 1e3, world)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    line = {"metric": "complex128 two-site DMRG sweeps/s (Fermi-Hubbard L=16, D=64, complex gauge)",
            "value": world * K / t_dev, "unit": "sweeps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * t_dev / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic",
            "config": {"workload": "fermi_hubbard_1d L=16 t=1 U=4 mu=0 (N,2Sz)=(16,0) D=64 maxiter=5 tol=1e-10, "
                                   "bond phases seed 5, start state seed 42 with entry phases seed 6",
                       "parallelism": f"replicas x{world}"},
            "clocks": clk.summary(), "gpu_launches": int(np.sum(la[W:W + K])), "energies": en.tolist()}
    if rank == 0 and not args.no_cpu_baseline:
        times, en_cpu, used = run_oracle_sweeps_for(Hr, psir, 1, os.cpu_count() or 1, D)
        line["cpu_baseline"] = {"value": 1.0 / float(times[0]), "unit": "sweeps/s", "cores": used, "kind": "port",
                                "sample": "first sweep of the real form of the problem (the C restatement has no "
                                          "complex path)"}
    if rank == 0:
        print(json.dumps(line), flush=True)


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
    ap.add_argument("--matvecs", type=int, default=1000, help="local-H applications timed in --mode localh")
    ap.add_argument("--orbitals", type=int, default=24, help="spatial orbitals of --mode molecular")
    ap.add_argument("--mol-vdim", type=int, default=512, help="bond dimension of --mode molecular")
    ap.add_argument("--mol-sweeps", type=int, default=10, help="sweeps of --mode molecular")
    ap.add_argument("--mol-precisions", default="fp64,bf16x3", help="runs of --mode molecular")
    ap.add_argument("--mol-profile", action="store_true", help="time every launch by kernel class in --mode molecular")
    ap.add_argument("--mol-oracle-sweeps", type=int, default=0,
                    help="sweeps of the CPU oracle from the same start state in --mode molecular (0: none)")
    ap.add_argument("--mode", default="full", choices=["full", "sweeps", "localh", "serve", "molecular", "singlesite", "complex"],
                    help="sweeps: only one device call of warmup+steps sweeps (for profiler captures), no JSON line; "
                         "localh: local-Hamiltonian microbenchmark (synthetic D=1024), its own JSON line; "
                         "serve: request stream of small and medium solves, serial vs concurrent solver threads; "
                         "molecular: spin-orbital molecular Hamiltonian (n=24, D=512), FP64 vs split-BF16; "
                         "singlesite: dmrg_singlesite on the Hubbard workload (D=256 fixed); "
                         "complex: complex128 two-site DMRG (Hubbard L=16, D=64, complex gauge)")
    ap.add_argument("--requests", type=int, default=128, help="requests of the --mode serve stream")
    ap.add_argument("--rate", type=float, default=50.0, help="Poisson arrival rate (1/s) of --mode serve")
    ap.add_argument("--workers", type=int, default=4, help="solver threads of --mode serve")
    ap.add_argument("--serve-precision", default="fp64", choices=sorted(PRECISIONS),
                    help="arithmetic of the concurrent solves of --mode serve (the serial baseline is FP64)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.mode == "sweeps":
        sweeps_only(args, local)
        return
    if args.mode == "localh":
        bench_local_h(args, world, rank, local)
        return
    if args.mode == "serve":
        bench_serve(args, world, rank, local)
        return
    if args.mode == "molecular":
        bench_molecular(args, world, rank, local)
        return
    if args.mode == "singlesite":
        bench_singlesite(args, world, rank, local)
        return
    if args.mode == "complex":
        bench_complex(args, world, rank, local)
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
