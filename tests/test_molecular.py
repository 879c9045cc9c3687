"""Spin-orbital molecular Hamiltonian MPO (host builder in libctgpu.so) against the reference's
construct_spin_molecular_hamiltonian_mpo_assembly(optimize=false) (src/operator/hamiltonian.c:2768),
and DMRG on it: oracle on the CPU here, the GPU path in the gpu-marked test."""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, workloads as wl
from conftest import golden
from helpers import overlap, run_gpu_dmrg, run_oracle_dmrg, same_structure


def _bond_dims(ch):
    return [t.dim_logical[0] for t in ch.tensors] + [ch.tensors[-1].dim_logical[3]]


@pytest.mark.parametrize("n", [1, 2, 4, 5])
def test_molecular_mpo_is_the_reference_operator(n):
    g = golden("spin_molecular_mpo.npz")
    ours = hm.spin_molecular(g[f"tkin{n}"], g[f"vint{n}"])
    ref = cs.chain_from_arrays(f"H{n}", g)
    assert _bond_dims(ours) == _bond_dims(ref)
    for a, b in zip(ours.tensors, ref.tensors):
        assert a.axis_dir == b.axis_dir
        for qa, qb in zip(a.qnums_logical, b.qnums_logical):
            assert sorted(qa.tolist()) == sorted(qb.tolist())
    ma, mb = hm.mpo_to_matrix(ours), hm.mpo_to_matrix(ref)
    assert np.abs(ma - mb).max() <= 1e-13 * np.abs(mb).max()


def test_molecular_mpo_dense_hamiltonian_small():
    """Independent check of the operator: the dense Jordan-Wigner Hamiltonian of 3 orbitals."""
    rng = np.random.default_rng(9)
    n = 3
    tk, vi = rng.standard_normal((n, n)), rng.standard_normal((n, n, n, n))
    nm = 2 * n
    z, u = np.diag([1.0, -1.0]), np.array([[0.0, 0.0], [1.0, 0.0]])
    cre = []
    for m in range(nm):
        op = np.ones((1, 1))
        for k in range(nm):
            op = np.kron(op, z if k < m else (u if k == m else np.eye(2)))
        cre.append(op)
    ann = [c.T for c in cre]
    h = np.zeros((4 ** n, 4 ** n))
    for i in range(n):
        for j in range(n):
            for s in range(2):
                h += tk[i, j] * cre[2 * i + s] @ ann[2 * j + s]
    for i in range(n):
        for j in range(n):
            for k in range(n):
                for l in range(n):
                    for s in range(2):
                        for t in range(2):
                            h += 0.5 * vi[i, j, k, l] * (cre[2 * i + s] @ cre[2 * j + t] @ ann[2 * l + t] @ ann[2 * k + s])
    got = hm.mpo_to_matrix(hm.spin_molecular(tk, vi))
    assert np.abs(got - h).max() <= 1e-12 * np.abs(h).max()


def test_molecular_mpo_structure_at_24_orbitals():
    """Bond quantum numbers (hence block structure) and stored entries of the 24-orbital workload
    equal the reference's: bond dimension up to 2 n^2 + 3 n + 2 = 1226."""
    g = golden("spin_molecular_mpo.npz")
    tk, vi = wl.molecular_integrals(24, 7)
    ch = hm.spin_molecular(tk, vi)
    assert max(_bond_dims(ch)) == 2 * 24 ** 2 + 3 * 24 + 2
    for i, t in enumerate(ch.tensors):
        assert np.array_equal(np.sort(np.asarray(t.qnums_logical[0], dtype=np.int32)), g[f"q24_bond{i}"])
        assert t.num_elements_blocks() == int(g[f"nnz24_site{i}"])


def test_oracle_dmrg_molecular_matches_reference(oracle_port):
    g = golden("dmrg_molecular_n6_D32.npz")
    L, D, sweeps, maxiter = [int(x) for x in g["params"]]
    H = cs.chain_from_arrays("H", g)
    psi0 = cs.chain_from_arrays("psi0", g)
    ret, en, ent, psi = run_oracle_dmrg(oracle_port, H, psi0, sweeps, maxiter, float(g["tol_split"]), D)
    assert ret == 0
    np.testing.assert_allclose(en, g["en_sweeps"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(ent, g["entropy"], rtol=0, atol=1e-10)
    assert same_structure(psi, cs.chain_from_arrays("psi", g))


@pytest.mark.gpu
def test_gpu_dmrg_molecular_matches_reference(gpu, oracle_port):
    """GPU dmrg_twosite on the MPO of this package's builder against the reference's run on its
    own MPO (same operator: energies agree to rounding)."""
    g = golden("dmrg_molecular_n6_D32.npz")
    L, D, sweeps, maxiter = [int(x) for x in g["params"]]
    H = hm.spin_molecular(g["tkin"], g["vint"])
    psi0 = cs.chain_from_arrays("psi0", g)
    ret, en, ent, psi = run_gpu_dmrg(gpu, H, psi0, sweeps, maxiter, float(g["tol_split"]), D)
    assert ret == 0
    np.testing.assert_allclose(en, g["en_sweeps"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(ent, g["entropy"], rtol=0, atol=1e-8)
    ref_psi = cs.chain_from_arrays("psi", g)
    assert same_structure(psi, ref_psi)
    assert abs(abs(overlap(oracle_port, psi, ref_psi)) - 1) < 1e-9
