"""Split-BF16 tcgen05 block GEMMs (ctgpu_set_precision(1)) against the FP64 oracle.

The split keeps 16 significant bits of each FP64 operand (a high and a low BF16 part) and sums
hi*hi + hi*lo + lo*hi in FP32 on the tensor cores, so a block product agrees with FP64 to about
2^-16 relative to sum_k |a_ik| |b_kj|. dmrg_twosite with this setting runs its last sweep in FP64.
"""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native
from conftest import golden
from helpers import c_bst, run_gpu_dmrg, run_oracle_dmrg, same_structure

pytestmark = pytest.mark.gpu

# relative to sum_k |a_ik||b_kj| for one block product
SPLIT_BF16_RTOL = 3e-5


@pytest.fixture
def split_bf16(gpu):
    old = native.set_precision(native.PRECISION_BF16X3)
    yield gpu
    native.set_precision(old)


def _abs_bst(t: cs.BlockSparse) -> cs.BlockSparse:
    a = cs.BlockSparse(t.dim_logical, t.axis_dir, t.qnums_logical)
    a.blocks = {k: np.abs(v) for k, v in t.blocks.items()}
    return a


def _dot(fn, s, axs, t, axt, nmult, check=True):
    cs_, ct_ = c_bst(s), c_bst(t)
    out = cs.BlockSparseTensor()
    ret = fn(C.byref(cs_), axs, C.byref(ct_), axt, nmult, C.byref(out))
    assert ret == 0 or not check
    r = cs.read_bst(out)
    for x in (out, cs_, ct_):
        cs.free_bst(x)
    return r


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("shape", ["small", "tiles"])
def test_split_bf16_dot_matches_oracle(split_bf16, oracle_port, seed, shape):
    rng = np.random.default_rng(500 + seed)
    # "tiles": blocks larger than one 128 x 64 tensor-core tile and K beyond one 64-wide stage
    lo, hi = (2, 14) if shape == "small" else (60, 200)
    nq = 2 if shape == "small" else 0
    dims = [int(x) for x in rng.integers(lo, hi, size=3)]
    qn = [rng.integers(-nq, nq + 1, size=d).astype(np.int32) for d in dims]
    axs, axt = seed % 2, (seed // 2) % 2
    # contracted axis: direction +1 on s, -1 on t
    if axs == 0:
        s = cs.BlockSparse((dims[1], dims[0]), (1, -1), [qn[1], qn[0]])
    else:
        s = cs.BlockSparse((dims[0], dims[1]), (1, 1), [qn[0], qn[1]])
    if axt == 0:
        t = cs.BlockSparse((dims[1], dims[2]), (-1, 1), [qn[1], qn[2]])
    else:
        t = cs.BlockSparse((dims[2], dims[1]), (1, -1), [qn[2], qn[1]])
    for x in (s, t):
        for idx in x.allowed:
            x.blocks[idx] = rng.standard_normal(x.block_shape(idx)) * 10.0 ** rng.uniform(-3, 3)
    got = _dot(split_bf16.ctgpu_block_sparse_tensor_dot, s, axs, t, axt, 1)
    ref = _dot(oracle_port.oracle_block_sparse_tensor_dot, s, axs, t, axt, 1, check=False)
    bound = _dot(oracle_port.oracle_block_sparse_tensor_dot, _abs_bst(s), axs, _abs_bst(t), axt, 1, check=False)
    assert got.dim_logical == ref.dim_logical and set(got.blocks) == set(ref.blocks)
    for k, v in ref.blocks.items():
        assert np.all(np.abs(got.blocks[k] - v) <= SPLIT_BF16_RTOL * bound.blocks[k] + 1e-300), k


def test_split_bf16_local_hamiltonian_matches_reference(split_bf16):
    g = golden("local_ops_hubbard_L8.npz")
    t = {k: cs.bst_from_arrays(k, g) for k in ["h2", "l", "r", "a", "b"]}
    c = {k: c_bst(v) for k, v in t.items()}
    out = cs.BlockSparseTensor()
    assert split_bf16.ctgpu_apply_local_hamiltonian(C.byref(c["a"]), C.byref(c["h2"]), C.byref(c["l"]),
                                                     C.byref(c["r"]), C.byref(out)) == 0
    got = cs.read_bst(out)
    cs.free_bst(out)
    num = sum(float(np.sum((got.blocks[k] - v) ** 2)) for k, v in t["b"].blocks.items())
    den = sum(float(np.sum(v ** 2)) for v in t["b"].blocks.values())
    # three chained products: a few 2^-16
    assert np.sqrt(num / den) < 1e-4
    for v in c.values():
        cs.free_bst(v)


def test_split_bf16_dmrg_final_fp64_sweep(split_bf16, oracle_port):
    """Mixed sweeps followed by one FP64 sweep land on the converged FP64 energy to 1e-8."""
    H = hm.fermi_hubbard_1d(12, 1.0, 4.0, 0.0)
    c = native.random_mps(12, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(12, 0), 48, 11)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    old = split_bf16.ctgpu_set_profiling(1, 0)
    try:
        r1, e1, s1, p1 = run_gpu_dmrg(split_bf16, H, psi0, 8, 5, 1e-10, 48)
    finally:
        split_bf16.ctgpu_set_profiling(old, 0)
    assert r1 == 0, native.last_error()
    prof = native.kernel_profile()
    # the tensor-core kernel ran in the mixed sweeps and the FP64 kernel in the final one
    assert prof["block_gemm_tc"]["launches"] > 0 and prof["block_gemm"]["launches"] > 0
    r2, e2, s2, p2 = run_oracle_dmrg(oracle_port, H, psi0, 8, 5, 1e-10, 48)
    assert r2 == 0
    # the reduced-precision sweeps agree with FP64 to the split's accuracy (the local Hamiltonian
    # and the environments are built from chained split-BF16 products; the energy is then not
    # variational and may fall slightly below the FP64 value) ...
    np.testing.assert_allclose(e1[:-1], e2[:-1], rtol=5e-4, atol=0)
    # ... and the final FP64 sweep reaches the FP64 energy
    assert abs(e1[-1] - e2[-1]) <= 1e-8
    assert native.last_stats()["matvecs"] > 0


def test_set_precision_rejects_unknown_values(gpu):
    assert native.lib().ctgpu_set_precision(7) < 0
    old = native.set_precision(native.PRECISION_FP64)
    assert native.set_precision(old) == native.PRECISION_FP64
