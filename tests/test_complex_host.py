"""Host side of the complex128 inputs: the bond-phase gauge keeps the operator, and the complex
fixtures hold complex tensors of the reference's block structure."""

import numpy as np

from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, workloads as wl
from conftest import golden


def test_bond_phase_gauge_keeps_the_operator():
    H = hm.fermi_hubbard_1d(3, 1.0, 4.0, 0.2)
    Hz = wl.complex_gauge(H, 5)
    assert all(t.dtype == cs.CT_DOUBLE_COMPLEX for t in Hz.tensors)
    assert max(np.abs(b.imag).max() for t in Hz.tensors for b in t.blocks.values()) > 0.1
    a, b = hm.mpo_to_matrix(H), hm.mpo_to_matrix(Hz)
    assert np.abs(a - b).max() <= 1e-14 * np.abs(a).max()
    assert np.abs(b - b.conj().T).max() <= 1e-14 * np.abs(b).max()


def test_complex_fixtures_round_trip():
    g = golden("dmrg_complex_hubbard_L6_D32.npz")
    for prefix in ("H", "psi0", "psi"):
        ch = cs.chain_from_arrays(prefix, g)
        assert all(t.dtype == cs.CT_DOUBLE_COMPLEX for t in ch.tensors)
        back = cs.chain_to_arrays(prefix, ch)
        for k, v in back.items():
            assert np.array_equal(np.asarray(g[k]), np.asarray(v)), k
