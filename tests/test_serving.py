"""Serving configuration: the seeded request stream (host) and concurrent solves (GPU) that must
give the same energies as the same solves one after another."""

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
