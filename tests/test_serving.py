"""Serving configuration: the seeded request stream (host) and concurrent solves (GPU) that must
give the same energies as the same solves one after another."""

import threading
import time

import numpy as np
import pytest

from chemtensor_gb300 import serving


def test_request_stream_is_seeded_and_in_range():
    a = serving.generate_requests(64, 10.0, seed=3)
    b = serving.generate_requests(64, 10.0, seed=3)
    assert [(r.arrival, r.model, r.nsites, r.max_vdim, r.param, r.seed) for r in a] == \
           [(r.arrival, r.model, r.nsites, r.max_vdim, r.param, r.seed) for r in b]
    assert all(8 <= r.nsites <= 48 and r.max_vdim in serving.BOND_DIMS for r in a)
    assert all((0.5 <= r.param <= 1.5) if r.model == "heisenberg" else (1.0 <= r.param <= 8.0) for r in a)
    t = np.array([r.arrival for r in a])
    assert np.all(np.diff(t) > 0)
    assert {r.model for r in a} == {"heisenberg", "hubbard"}


@pytest.mark.gpu
def test_concurrent_solves_match_serial():
    reqs = [r for r in serving.generate_requests(40, 0.0, seed=11) if r.max_vdim <= 64 and r.nsites <= 24][:6]
    assert len(reqs) >= 3
    serial = serving.SolverPool(workers=1, sweeps=2).run(reqs)
    conc = serving.SolverPool(workers=3, sweeps=2).run(reqs)
    assert all(r.ret == 0 for r in serial + conc), [r.error for r in serial + conc]
    for a, b in zip(serial, conc):
        # each solve is deterministic: the same energy whatever runs beside it
        assert a.energy == b.energy
    assert len({r.worker for r in conc}) > 1


@pytest.mark.gpu
def test_concurrent_mixed_precision_solves_match_serial():
    """Reduced-precision solves (split-BF16 matvecs where the autotuner puts them on the tensor cores,
    final sweep FP64) give the same energy alone and in the mix: every kernel is deterministic and
    the autotuner's picks are process-wide, so solves running side by side take the same paths."""
    from chemtensor_gb300 import native
    reqs = [r for r in serving.generate_requests(60, 0.0, seed=13) if r.max_vdim <= 64 and r.nsites <= 24][:6]
    assert len(reqs) >= 3
    p = native.PRECISION_BF16X3
    serial = serving.SolverPool(workers=1, sweeps=2, precision=p).run(reqs)
    conc = serving.SolverPool(workers=3, sweeps=2, precision=p, prefetch=4).run(reqs)
    assert all(r.ret == 0 for r in serial + conc), [r.error for r in serial + conc]
    for a, b in zip(serial, conc):
        assert a.energy == b.energy
    assert len({r.worker for r in conc}) > 1


def test_admission_keeps_solves_in_flight_within_the_budget():
    """Host logic of admission by estimated HBM footprint: a fake solve records how many bytes were
    admitted while it ran; the total never exceeds the budget, and a request larger than the whole
    budget still runs (alone)."""
    reqs = serving.generate_requests(24, 0.0, seed=5)
    est = {r.rid: serving.estimate_footprint(r) for r in reqs}
    budget = sorted(est.values())[len(est) // 2] * 2          # about two median solves at a time
    lock = threading.Lock()
    live, seen = {}, []

    def fake_solve(req, res, lib):
        with lock:
            live[req.rid] = min(est[req.rid], budget)
            seen.append(sum(live.values()))
        time.sleep(0.002)
        with lock:
            del live[req.rid]
        res.ret, res.energy = 0, float(req.rid)

    pool = serving.SolverPool(workers=6, hbm_budget=budget, solve=fake_solve)
    out = pool.run(reqs)
    assert all(r.ret == 0 for r in out)
    assert max(seen) <= budget and pool.admission_peak <= budget
    assert any(v > budget for v in est.values()) or max(seen) > 0


def test_footprint_estimate_grows_with_size():
    small = serving.Request(0, 0.0, "hubbard", 8, 16, 4.0, 1)
    big = serving.Request(1, 0.0, "hubbard", 48, 256, 4.0, 1)
    assert 0 < serving.estimate_footprint(small) < serving.estimate_footprint(big)
    # the dense bound of a D = 256, L = 48 Hubbard solve stays far below one GPU's HBM
    assert serving.estimate_footprint(big) < 4 << 30
