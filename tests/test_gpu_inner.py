"""mpo_inner_product (<chi|H|psi>, src/algorithm/chain_ops.c:274-317) on the device, against dense
vectors and operators, and as the check of a DMRG energy without a host round trip."""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native, workloads as wl
from helpers import run_gpu_dmrg
from test_gpu_complex import mps_vector

pytestmark = pytest.mark.gpu


def _random(L, D, seed, sector):
    c = native.random_mps(L, 4, hm.HUBBARD_QSITE, sector, D, seed)
    out = cs.read_mps(c)
    cs.free_mps(c)
    return out


def _inner(gpu, chi, H, psi, cplx=False):
    cc, ch, cp = cs.make_c_mps(chi), cs.make_c_mpo(H), cs.make_c_mps(psi)
    out = (C.c_double * 2)()
    ret = gpu.ctgpu_mpo_inner_product(C.byref(cc), C.byref(ch), C.byref(cp), out)
    for x in (cc, cp):
        cs.free_mps(x)
    cs.free_mpo(ch)
    assert ret == 0, native.last_error()
    return complex(out[0], out[1]) if cplx else out[0]


def test_mpo_inner_product_matches_dense(gpu):
    L = 5
    sector = hm.encode_quantum_number_pair(L, 1)
    H = hm.fermi_hubbard_1d(L, 1.0, 4.0, 0.3)
    chi, psi = _random(L, 12, 3, sector), _random(L, 12, 4, sector)
    ref = mps_vector(chi) @ hm.mpo_to_matrix(H) @ mps_vector(psi)
    got = _inner(gpu, chi, H, psi)
    assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref))


def test_mpo_inner_product_complex_matches_dense(gpu):
    L = 4
    sector = hm.encode_quantum_number_pair(L, 0)
    H = wl.complex_gauge(hm.fermi_hubbard_1d(L, 1.0, 2.0, 0.0), 9)
    chi = wl.complex_gauge(_random(L, 8, 5, sector), 10, entry_phases=True)
    psi = wl.complex_gauge(_random(L, 8, 6, sector), 11, entry_phases=True)
    ref = np.vdot(mps_vector(chi), hm.mpo_to_matrix(H) @ mps_vector(psi))
    got = _inner(gpu, chi, H, psi, cplx=True)
    assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref))


def test_energy_of_dmrg_result(gpu):
    """<psi|H|psi> of the returned (normalised) state equals the last sweep's energy: the final
    local eigenproblem's Ritz value is the state's energy to the Lanczos accuracy."""
    L, D = 10, 32
    H = hm.fermi_hubbard_1d(L, 1.0, 4.0, 0.0)
    psi0 = _random(L, D, 7, hm.encode_quantum_number_pair(L, 0))
    ret, en, ent, psi = run_gpu_dmrg(gpu, H, psi0, 4, 5, 1e-10, D)
    assert ret == 0
    e = _inner(gpu, psi, H, psi)
    assert abs(e - en[-1]) <= 1e-8 * abs(en[-1]), (e, en[-1])
