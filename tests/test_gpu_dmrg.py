"""dmrg_twosite and dmrg_singlesite on the GPU through the C ABI, against the reference's own results."""

import ctypes as C

import numpy as np
import pytest

import chemtensor_gb300 as ctg
from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native
from conftest import golden
from helpers import overlap, run_gpu_dmrg, run_oracle_dmrg, same_structure

pytestmark = pytest.mark.gpu

CASES = ["dmrg_heisenberg_L20_D32.npz", "dmrg_heisenberg_L10_D16.npz",
         "dmrg_hubbard_L8_D32.npz", "dmrg_hubbard_L12_D48.npz"]


@pytest.mark.parametrize("case", CASES)
def test_dmrg_matches_reference(gpu, oracle_port, case):
    g = golden(case)
    L, D, sweeps, maxiter = [int(x) for x in g["params"]]
    H = cs.chain_from_arrays("H", g)
    psi0 = cs.chain_from_arrays("psi0", g)
    ret, en, ent, psi = run_gpu_dmrg(gpu, H, psi0, sweeps, maxiter, float(g["tol_split"]), D)
    assert ret == 0, native.last_error()
    # energies within 1e-10 of the reference, bond structure and quantum numbers bit-exact
    np.testing.assert_allclose(en, g["en_sweeps"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(ent, g["entropy"], rtol=0, atol=1e-8)
    ref_psi = cs.chain_from_arrays("psi", g)
    assert same_structure(psi, ref_psi)
    # same state up to a global sign (gauge-invariant), normalised
    assert abs(abs(overlap(oracle_port, psi, ref_psi)) - 1) < 1e-9
    assert abs(overlap(oracle_port, psi, psi) - 1) < 1e-12


def test_dmrg_with_package_hamiltonian_matches_oracle(gpu, oracle_port):
    H = hm.fermi_hubbard_1d(16, 1.0, 4.0, 0.0)
    c = native.random_mps(16, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(16, 0), 64, 42)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    r1, e1, s1, p1 = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 64)
    r2, e2, s2, p2 = run_oracle_dmrg(oracle_port, H, psi0, 2, 5, 1e-10, 64)
    assert r1 == 0 and r2 == 0
    np.testing.assert_allclose(e1, e2, rtol=0, atol=1e-10)
    np.testing.assert_allclose(s1, s2, rtol=0, atol=1e-8)
    assert same_structure(p1, p2)


_GRID_FORM_SCRIPT = r"""
import json, sys
sys.path.insert(0, "tests")
from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native
from helpers import run_gpu_dmrg
H = hm.fermi_hubbard_1d(16, 1.0, 4.0, 0.0)
c = native.random_mps(16, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(16, 0), 64, 42)
psi0 = cs.read_mps(c)
cs.free_mps(c)
ret, en, ent, psi = run_gpu_dmrg(native.lib(), H, psi0, 2, 5, 1e-10, 64)
print(json.dumps({"ret": ret, "en": list(en), "ent": list(ent)}))
"""


def test_lanczos_grid_and_cluster_forms_match_oracle(gpu, oracle_port):
    """The Lanczos vector kernels run as one thread-block cluster for vectors that fit and as a
    cooperative grid otherwise: the same solve with every vector forced onto the grid form (in a
    child process, CTGPU_LZ_CLUSTER_MAX_N=0) and with the default choice (cluster form at this size)
    both match the oracle."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CTGPU_LZ_CLUSTER_MAX_N="0")
    r = subprocess.run([sys.executable, "-c", _GRID_FORM_SCRIPT], cwd=root, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    grid = json.loads(r.stdout.strip().splitlines()[-1])
    H = hm.fermi_hubbard_1d(16, 1.0, 4.0, 0.0)
    c = native.random_mps(16, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(16, 0), 64, 42)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    r1, e1, s1, _ = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 64)
    r2, e2, s2, _ = run_oracle_dmrg(oracle_port, H, psi0, 2, 5, 1e-10, 64)
    assert r1 == 0 and r2 == 0 and grid["ret"] == 0
    np.testing.assert_allclose(e1, e2, rtol=0, atol=1e-10)
    np.testing.assert_allclose(grid["en"], e2, rtol=0, atol=1e-10)
    np.testing.assert_allclose(grid["ent"], s2, rtol=0, atol=1e-8)


def test_launch_without_programmatic_dependence_gives_the_same_bits(gpu):
    """The sweep's kernels are launched with programmatic dependent launch (each waits for its
    predecessor on the device before touching memory); with it switched off (child process,
    CTGPU_PDL=0) the same solve gives bit-identical energies and entropies."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CTGPU_PDL="0")
    r = subprocess.run([sys.executable, "-c", _GRID_FORM_SCRIPT], cwd=root, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    off = json.loads(r.stdout.strip().splitlines()[-1])
    H = hm.fermi_hubbard_1d(16, 1.0, 4.0, 0.0)
    c = native.random_mps(16, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(16, 0), 64, 42)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    ret, en, ent, _ = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 64)
    assert ret == 0 and off["ret"] == 0
    assert list(en) == off["en"] and list(ent) == off["ent"]


@pytest.mark.parametrize("L,D,seed", [(10, 8, 268), (14, 8, 71)])
def test_dmrg_zero_norm_start_state_matches_oracle(gpu, oracle_port, L, D, seed):
    """A seeded random start state with a site tensor that has no allowed block (mismatching quantum
    numbers, norm zero): the reference warns and carries on (its right-normalisation leaves
    isometries), and so must the GPU path. A product with no output block packs no descriptors."""
    H = hm.fermi_hubbard_1d(L, 1.0, 4.0, 0.0)
    c = native.random_mps(L, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(L, 0), D, seed)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    assert any(len(t.blocks) == 0 for t in psi0.tensors)
    r1, e1, s1, p1 = run_gpu_dmrg(gpu, H, psi0, 3, 5, 1e-10, D)
    r2, e2, s2, p2 = run_oracle_dmrg(oracle_port, H, psi0, 3, 5, 1e-10, D)
    assert r1 == r2 == 0, native.last_error()
    np.testing.assert_allclose(e1, e2, rtol=0, atol=1e-10)
    assert same_structure(p1, p2)


def test_dmrg_hubbard_L32_D256_matches_oracle(gpu, oracle_port):
    """The headline workload (Fermi-Hubbard L=32, t=1, U=4, (N, 2Sz) = (32, 0), D=256, maxiter 5,
    tol 1e-10, seeded start state 42), two sweeps, against the oracle on the host cores: energies
    within 1e-10, every bond's quantum numbers bit-exact, the retained singular values of every bond
    within 1e-8 relative, |<psi_gpu|psi_oracle>| = 1 within 1e-9."""
    import oracle
    L, D, sweeps = 32, 256, 2
    H = hm.fermi_hubbard_1d(L, 1.0, 4.0, 0.0)
    c = native.random_mps(L, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(L, 0), D, 42)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    r1, e1, s1, p1 = run_gpu_dmrg(gpu, H, psi0, sweeps, 5, 1e-10, D)
    assert r1 == 0, native.last_error()
    st = native.last_stats()
    sig_gpu = [native.bond_singular_values(b) for b in range(L - 1)]
    oracle_port.oracle_set_num_threads(0)
    r2, e2, s2, p2 = run_oracle_dmrg(oracle_port, H, psi0, sweeps, 5, 1e-10, D)
    assert r2 == 0
    sig_orc = [oracle.bond_sigma(oracle_port, b) for b in range(L - 1)]
    np.testing.assert_allclose(e1, e2, rtol=0, atol=1e-10)
    np.testing.assert_allclose(s1, s2, rtol=0, atol=1e-8)
    assert same_structure(p1, p2)
    assert max(t.dim_logical[2] for t in p1.tensors) == D
    # cuts that fell between singular values equal to rounding (the Hubbard chain's spin multiplets):
    # reported; the kept sets above agree all the same
    print(f"near-ties at the bond-dimension cut: {st['near_ties']}")
    for b in range(L - 1):
        assert sig_gpu[b] is not None and sig_orc[b] is not None, b
        assert len(sig_gpu[b]) == len(sig_orc[b]), b
        np.testing.assert_allclose(sig_gpu[b], sig_orc[b], rtol=1e-8, atol=0, err_msg=f"bond {b}")
    assert abs(abs(overlap(oracle_port, p1, p2)) - 1) < 1e-9


def test_python_entry_point_mirrors_reference_binding(gpu):
    H = hm.heisenberg_xxz_1d(10, 1.0, 1.0, 0.0)
    psi, en, ent = ctg.dmrg(H, num_sweeps=3, maxiter_lanczos=5, tol_split=1e-10, max_vdim=16, qnum_sector=0, rng_seed=7)
    assert len(en) == 3 and len(ent) == 9
    assert en[-1] < -4.2
    with pytest.raises(ValueError):
        ctg.dmrg(H, num_sweeps=0)


def test_invalid_arguments_return_error_code(gpu):
    H = hm.heisenberg_xxz_1d(6, 1.0, 1.0, 0.0)
    cH = cs.make_c_mpo(H)
    p = native.random_mps(5, 2, [1, -1], 0, 8, 1)       # wrong length
    en, ent = np.zeros(2), np.zeros(5)
    assert gpu.dmrg_twosite(C.byref(cH), 2, 5, 1e-10, 8, C.byref(p), en.ctypes.data, ent.ctypes.data) == -5
    assert "nsites" in native.last_error()
    cs.free_mps(p)
    p = native.random_mps(6, 2, [1, -1], 0, 8, 1)
    assert gpu.dmrg_twosite(C.byref(cH), 2, 999, 1e-10, 8, C.byref(p), en.ctypes.data, ent.ctypes.data) == -5
    cs.free_mps(p)
    cs.free_mpo(cH)


def test_repeated_calls_are_deterministic(gpu):
    g = golden("dmrg_hubbard_L8_D32.npz")
    H = cs.chain_from_arrays("H", g)
    psi0 = cs.chain_from_arrays("psi0", g)
    a = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 32)
    b = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 32)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("case", ["dmrg1_heisenberg_L12_D16.npz", "dmrg1_hubbard_L8_D24.npz"])
def test_dmrg_singlesite_matches_reference(gpu, oracle_port, case):
    g = golden(case)
    L, D, sweeps, maxiter = [int(x) for x in g["params"]]
    H = cs.chain_from_arrays("H", g)
    psi0 = cs.chain_from_arrays("psi0", g)
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en = np.zeros(sweeps)
    ret = gpu.dmrg_singlesite(C.byref(cH), sweeps, maxiter, C.byref(cP), en.ctypes.data)
    psi = cs.read_mps(cP)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    assert ret == 0
    np.testing.assert_allclose(en, g["en_sweeps"], rtol=0, atol=1e-10)
    ref_psi = cs.chain_from_arrays("psi", g)
    assert same_structure(psi, ref_psi)
    assert abs(abs(overlap(oracle_port, psi, ref_psi)) - 1) < 1e-9
    assert abs(overlap(oracle_port, psi, psi) - 1) < 1e-12
