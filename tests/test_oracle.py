"""The C oracle against the reference's own outputs (golden fixtures) - CPU only."""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs
from conftest import golden
from helpers import assert_bst_close, c_bst, overlap, run_oracle_dmrg, same_structure

DMRG_CASES = ["dmrg_heisenberg_L20_D32.npz", "dmrg_heisenberg_L10_D16.npz",
              "dmrg_hubbard_L8_D32.npz", "dmrg_hubbard_L12_D48.npz"]


@pytest.mark.parametrize("case", DMRG_CASES)
def test_oracle_dmrg_matches_reference(oracle_port, case):
    g = golden(case)
    L, D, sweeps, maxiter = [int(x) for x in g["params"]]
    H = cs.chain_from_arrays("H", g)
    psi0 = cs.chain_from_arrays("psi0", g)
    ret, en, ent, psi = run_oracle_dmrg(oracle_port, H, psi0, sweeps, maxiter, float(g["tol_split"]), D)
    assert ret == 0
    np.testing.assert_allclose(en, g["en_sweeps"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(ent, g["entropy"], rtol=0, atol=1e-10)
    ref_psi = cs.chain_from_arrays("psi", g)
    assert same_structure(psi, ref_psi)
    assert abs(abs(overlap(oracle_port, psi, ref_psi)) - 1) < 1e-10
    assert abs(overlap(oracle_port, psi, psi) - 1) < 1e-12


@pytest.mark.parametrize("case", ["local_ops_heisenberg_L12.npz", "local_ops_hubbard_L8.npz"])
def test_oracle_local_ops_match_reference(oracle_port, case):
    g = golden(case)
    t = {k: cs.bst_from_arrays(k, g) for k in ["h2", "l", "r", "a", "b", "lnext", "rnext", "A", "B", "W", "W1"]}
    c = {k: c_bst(v) for k, v in t.items()}
    out = cs.BlockSparseTensor()
    oracle_port.oracle_apply_local_hamiltonian(C.byref(c["a"]), C.byref(c["h2"]), C.byref(c["l"]), C.byref(c["r"]), C.byref(out))
    assert_bst_close(cs.read_bst(out), t["b"], 1e-13)
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(out))
    out = cs.BlockSparseTensor()
    oracle_port.oracle_contraction_operator_step_left(C.byref(c["A"]), C.byref(c["A"]), C.byref(c["W"]), C.byref(c["l"]), C.byref(out))
    assert_bst_close(cs.read_bst(out), t["lnext"], 1e-13)
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(out))
    out = cs.BlockSparseTensor()
    oracle_port.oracle_contraction_operator_step_right(C.byref(c["B"]), C.byref(c["B"]), C.byref(c["W1"]), C.byref(c["r"]), C.byref(out))
    assert_bst_close(cs.read_bst(out), t["rnext"], 1e-13)
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(out))
    for v in c.values():
        cs.free_bst(v)


def _retained(port, sigma, tol, max_vdim):
    s = np.ascontiguousarray(sigma, dtype=np.float64)
    ind = np.zeros(max(len(s), 1), dtype=np.int64)
    nrm, ent, tol_eff = C.c_double(), C.c_double(), C.c_double()
    n = port.oracle_retained_bond_indices(s.ctypes.data, len(s), tol, 1, max_vdim, ind.ctypes.data,
                                          C.byref(nrm), C.byref(ent), C.byref(tol_eff))
    return list(ind[:n]), nrm.value, ent.value, tol_eff.value


def test_oracle_truncation_rules(oracle_port):
    # truncation.c:110-223: cumulative squared weights from the smallest value, relative threshold
    s = np.array([0.5, 1e-7, 0.8, 0.3, 1e-3])
    ind, nrm, ent, tol_eff = _retained(oracle_port, s, 1e-10, 10)
    assert ind == [0, 2, 3, 4]                      # 1e-7 squared is below 1e-10 of the total
    assert abs(nrm - np.linalg.norm(s[[0, 2, 3, 4]])) < 1e-15
    p = s[[0, 2, 3, 4]] ** 2 / nrm ** 2
    assert abs(ent + np.sum(p * np.log(p))) < 1e-14
    ind, _, _, tol_eff = _retained(oracle_port, s, 1e-10, 2)   # max_vdim cut keeps the two largest
    assert ind == [0, 2] and tol_eff > 1e-10
    assert _retained(oracle_port, np.zeros(4), 1e-10, 4)[0] == []   # all zero: nothing retained
    ind, _, _, _ = _retained(oracle_port, np.array([0.6, 0.6, 0.6, 0.1]), 0.0, 2)
    assert ind == [1, 2]                            # exact ties: the later indices carry larger sums


def test_oracle_lanczos_exact_in_full_krylov_space(oracle_port):
    rng = np.random.default_rng(3)
    n = 12
    a = rng.standard_normal((n, n))
    h = np.ascontiguousarray(a + a.T)
    v0 = rng.standard_normal(n)
    lam, u = C.c_double(), np.zeros(n)
    assert oracle_port.oracle_lanczos_dense(n, h.ctypes.data, v0.ctypes.data, n, C.byref(lam), u.ctypes.data) == 0
    w = np.linalg.eigvalsh(h)
    assert abs(lam.value - w[0]) < 1e-10
    assert np.linalg.norm(h @ u - lam.value * u) < 1e-8


QR_TAGS = ["m0", "m1", "m2", "m3", "m4"]


@pytest.mark.parametrize("tag", QR_TAGS)
def test_oracle_qr_rq_match_reference(oracle_port, tag):
    """block_sparse_tensor_qr / _rq restated (dgeqrf / dgerqf per block) against the reference's factors."""
    g = golden("qr_rq_blocks.npz")
    a = c_bst(cs.bst_from_arrays(tag, g))
    q, r = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    assert oracle_port.oracle_block_sparse_tensor_qr(C.byref(a), C.byref(q), C.byref(r)) == 0
    assert_bst_close(cs.read_bst(q), cs.bst_from_arrays(tag + "_qr_q", g), 1e-13)
    assert_bst_close(cs.read_bst(r), cs.bst_from_arrays(tag + "_qr_r", g), 1e-13)
    r2, q2 = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    assert oracle_port.oracle_block_sparse_tensor_rq(C.byref(a), C.byref(r2), C.byref(q2)) == 0
    assert_bst_close(cs.read_bst(r2), cs.bst_from_arrays(tag + "_rq_r", g), 1e-13)
    assert_bst_close(cs.read_bst(q2), cs.bst_from_arrays(tag + "_rq_q", g), 1e-13)
    for x in (q, r, r2, q2):
        oracle_port.oracle_delete_block_sparse_tensor(C.byref(x))
    cs.free_bst(a)


@pytest.mark.parametrize("case", ["dmrg1_heisenberg_L12_D16.npz", "dmrg1_hubbard_L8_D24.npz"])
def test_oracle_dmrg_singlesite_matches_reference(oracle_port, case):
    g = golden(case)
    L, D, sweeps, maxiter = [int(x) for x in g["params"]]
    H = cs.chain_from_arrays("H", g)
    psi0 = cs.chain_from_arrays("psi0", g)
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en = np.zeros(sweeps)
    ret = oracle_port.oracle_dmrg_singlesite(C.byref(cH), sweeps, maxiter, C.byref(cP), en.ctypes.data)
    psi = cs.read_mps(cP)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    assert ret == 0
    np.testing.assert_allclose(en, g["en_sweeps"], rtol=0, atol=1e-12)
    ref_psi = cs.chain_from_arrays("psi", g)
    assert same_structure(psi, ref_psi)
    assert abs(abs(overlap(oracle_port, psi, ref_psi)) - 1) < 1e-10
    assert abs(overlap(oracle_port, psi, psi) - 1) < 1e-12
