"""A small DMRG solve service on one GPU: seeded request streams and a pool of solver threads.

Each request is a ground-state search (two-site DMRG through the C-ABI ``dmrg_twosite``) for a 1D
Heisenberg XXZ or Fermi-Hubbard chain. Worker threads take requests in arrival order; every thread
owns its own execution context in libctgpu.so (stream, memory pool, plan cache), so solves of
different threads run side by side on the GPU while each thread's solve stays sequential. The
library's per-call state (device, precision, last error, statistics) is thread-local.

Admission: before a thread starts a solve, the request's HBM footprint is estimated from its length,
bond dimension, local dimension and MPO bond dimension (an upper bound that ignores block
sparsity: environments, MPS, merged MPO pairs and the local-problem intermediates), and the solve
waits until the estimates of the solves in flight plus its own fit the pool's budget (by default
half of the device memory that is free when the pool starts). A request larger than the whole
budget runs alone.

Inputs: with `prefetch`, a producer thread builds every request's MPO and seeded start state (as the C
structs dmrg_twosite takes) ahead of the solvers, in arrival order, so that input building does not
sit on a solver's critical path.

Request mix (the serving configuration of the two-site DMRG scope): Heisenberg with anisotropy
Delta ~ U[0.5, 1.5] or Hubbard with U ~ U[1, 8] (t = 1, half filling), length L ~ U{8..48}, bond
dimension D in {16, 32, 64, 128, 256}, Poisson arrivals; every parameter drawn from one seeded
generator.
"""

from __future__ import annotations

import ctypes as C
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import ctstructs as cs
from . import hamiltonians as hm
from . import native

BOND_DIMS = (16, 32, 64, 128, 256)


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the stream
    model: str              # "heisenberg" or "hubbard"
    nsites: int
    max_vdim: int
    param: float            # Delta (Heisenberg) or U (Hubbard)
    seed: int


@dataclass
class Result:
    rid: int
    arrival: float
    start: float = 0.0
    end: float = 0.0
    energy: float = float("nan")
    ret: int = 0
    worker: int = -1
    error: str = ""

    @property
    def latency(self) -> float:
        return self.end - self.arrival


def generate_requests(n: int, rate: float, seed: int) -> list[Request]:
    """n requests with exponential inter-arrival times of mean 1 / rate (seconds)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate)) if rate > 0 else 0.0
        hub = bool(rng.random() < 0.5)
        nsites = int(rng.integers(8, 49))
        d = int(rng.choice(BOND_DIMS))
        param = float(rng.uniform(1.0, 8.0)) if hub else float(rng.uniform(0.5, 1.5))
        out.append(Request(i, t, "hubbard" if hub else "heisenberg", nsites, d, param, int(rng.integers(1, 2**31))))
    return out


MPO_BOND_DIM = {"heisenberg": 5, "hubbard": 6}


def estimate_footprint(req: Request, sweeps_buffers: int = 3) -> int:
    """Upper bound (bytes) of the device memory of one two-site DMRG solve, without block sparsity:
    left and right environments L x D x Dw x D, the MPS L x D x d x D, merged MPO pairs
    (L - 1) x Dw^2 x d^4, and `sweeps_buffers` two-site intermediates D x d^2 x Dw x D."""
    d = 4 if req.model == "hubbard" else 2
    dw = MPO_BOND_DIM[req.model]
    L, D = req.nsites, req.max_vdim
    env = 2 * L * D * dw * D
    mps = L * D * d * D
    h2 = (L - 1) * dw * dw * d ** 4
    inter = sweeps_buffers * D * d * d * dw * D
    return 8 * (env + mps + h2 + inter)


class Admission:
    """Byte budget shared by the solver threads: acquire blocks until the request fits."""

    def __init__(self, budget: int):
        self.budget = int(budget)
        self.in_use = 0
        self.peak = 0
        self.cv = threading.Condition()

    def acquire(self, nbytes: int) -> int:
        take = min(int(nbytes), self.budget)     # a request larger than the budget runs alone
        with self.cv:
            while self.in_use + take > self.budget:
                self.cv.wait()
            self.in_use += take
            self.peak = max(self.peak, self.in_use)
        return take

    def release(self, take: int) -> None:
        with self.cv:
            self.in_use -= take
            self.cv.notify_all()


def device_free_bytes(device: int) -> int:
    import ctypes as C
    free, total = C.c_size_t(), C.c_size_t()
    if native.lib().ctgpu_device_memory(device, C.byref(free), C.byref(total)) != 0:
        raise RuntimeError(native.last_error())
    return int(free.value)


def build_problem(req: Request):
    """MPO and seeded random start state of a request (host side), as Python chains."""
    cH, cP = build_problem_c(req)
    H, psi = cs.read_mpo(cH), cs.read_mps(cP)
    cs.free_mpo(cH)
    cs.free_mps(cP)
    return H, psi


def build_problem_c(req: Request):
    """MPO and seeded random start state of a request as the C structs dmrg_twosite takes: the start
    state comes straight from the library's generator (no round trip through Python objects)."""
    # half filling / smallest total spin: 2 Sz = L mod 2
    sz2 = req.nsites % 2
    if req.model == "hubbard":
        H = hm.fermi_hubbard_1d(req.nsites, 1.0, req.param, 0.0)
        c = native.random_mps(req.nsites, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(req.nsites, sz2),
                              req.max_vdim, req.seed)
    else:
        H = hm.heisenberg_xxz_1d(req.nsites, 1.0, req.param, 0.0)
        c = native.random_mps(req.nsites, 2, [1, -1], sz2, req.max_vdim, req.seed)
    return cs.make_c_mpo(H), c


@dataclass
class SolverPool:
    """Replays a request stream against `workers` solver threads on one GPU."""
    workers: int = 4
    device: int = 0
    sweeps: int = 2
    maxiter: int = 5
    tol: float = 1e-10
    precision: int = native.PRECISION_FP64
    hbm_budget: int | None = None       # bytes; None: half of the free device memory at start
    solve: object = None                # the solve function (request, result, lib); None: DMRG
    results: list = field(default_factory=list)
    admission_peak: int = 0

    prefetch: int = 0                   # problems built ahead by a producer thread (0: built by the solver)

    def _solve(self, req: Request, res: Result, lib, problem=None):
        cH, cP = problem if problem is not None else build_problem_c(req)
        en = np.zeros(self.sweeps)
        ent = np.zeros(max(req.nsites - 1, 1))
        try:
            res.ret = lib.dmrg_twosite(C.byref(cH), self.sweeps, self.maxiter, self.tol, req.max_vdim, C.byref(cP),
                                       en.ctypes.data, ent.ctypes.data)
            res.energy = float(en[-1])
            if res.ret != 0:
                res.error = native.last_error()
        finally:
            cs.free_mps(cP)
            cs.free_mpo(cH)

    def run(self, requests: list[Request]) -> list[Result]:
        lib = native.lib() if self.solve is None else None
        solve = self.solve or self._solve
        budget = self.hbm_budget if self.hbm_budget is not None else device_free_bytes(self.device) // 2
        adm = Admission(budget)
        ordered = sorted(requests, key=lambda r: r.arrival)
        results = {r.rid: Result(r.rid, r.arrival) for r in requests}
        errors = []
        # requests in arrival order; with prefetch, a producer thread builds each request's MPO and start
        # state ahead of the solvers (bounded queue), so that input building leaves their critical path
        q: queue.Queue = queue.Queue(maxsize=self.prefetch if (self.prefetch and lib is not None) else 0)
        producer = None
        if self.prefetch and lib is not None:
            def produce():
                for r in ordered:
                    try:
                        q.put((r, build_problem_c(r)))
                    except Exception as e:   # the solver records it
                        q.put((r, e))
                for _ in range(self.workers):
                    q.put(None)
            producer = threading.Thread(target=produce, daemon=True)
        else:
            for r in ordered:
                q.put((r, None))
            for _ in range(self.workers):
                q.put(None)
        t0 = time.perf_counter()

        def worker(wid: int):
            if lib is not None:
                lib.ctgpu_set_device(self.device)
                lib.ctgpu_set_precision(self.precision)
            while True:
                item = q.get()
                if item is None:
                    return
                req, problem = item
                wait = req.arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(wait)
                res = results[req.rid]
                res.worker = wid
                take = adm.acquire(estimate_footprint(req))
                res.start = time.perf_counter() - t0
                try:
                    if isinstance(problem, Exception):
                        raise problem
                    if problem is not None:
                        solve(req, res, lib, problem)
                    else:
                        solve(req, res, lib)
                except Exception as e:  # recorded, the stream goes on
                    res.ret = -99
                    res.error = str(e)
                    errors.append(e)
                finally:
                    adm.release(take)
                res.end = time.perf_counter() - t0

        threads = [threading.Thread(target=worker, args=(i,), daemon=True) for i in range(self.workers)]
        if producer is not None:
            producer.start()
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        self.results = [results[r.rid] for r in requests]
        self.admission_peak = adm.peak
        return self.results


def summarize(results: list[Result]) -> dict:
    lat = np.array([r.latency for r in results if r.ret == 0])
    span = max(r.end for r in results) - min(r.arrival for r in results) if results else 0.0
    ok = int(np.sum([r.ret == 0 for r in results]))
    return {
        "requests": len(results), "solved": ok, "failed": len(results) - ok,
        "solves_per_s": ok / span if span > 0 else None,
        "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
        "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
        "mean_ms": float(lat.mean() * 1e3) if lat.size else None,
        "makespan_s": span,
    }
