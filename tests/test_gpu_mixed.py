"""Reduced-precision tcgen05 block GEMMs (ctgpu_set_precision(1|2|3)) against the FP64 oracle.

Formats and their accuracy, relative to sum_k |a_ik| |b_kj| of one block product (FP32 accumulation
on the tensor cores in every case):
  1 split-BF16 (hi + lo, 3 products)          keeps 16 bits of each operand: about 2^-16
  2 TF32 (one product)                        keeps 11 bits: about 2^-11
  3 three-part split-BF16 (hi + mid + lo, 6)  keeps the 24 bits of FP32: about 2^-23 on short
                                              contractions; on long ones the FP32 accumulation
                                              bounds both BF16 forms alike
dmrg_twosite with any of them runs its last sweep in FP64. Every tile width of the tensor-core
GEMM (64, 128, 256 columns) is exercised.
"""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native
from conftest import golden
from helpers import c_bst, run_gpu_dmrg, run_oracle_dmrg

pytestmark = pytest.mark.gpu

# per-product tolerance relative to sum_k |a_ik||b_kj|
DOT_RTOL = {native.PRECISION_BF16X3: 3e-5, native.PRECISION_TF32: 3e-3, native.PRECISION_BF16X6: 2e-6}
# relative Frobenius error of the local Hamiltonian (three chained products; on long contractions the
# FP32 accumulation on the tensor cores, not the operand split, sets the error of both BF16 forms)
LOCAL_H_RTOL = {native.PRECISION_BF16X3: 1e-4, native.PRECISION_TF32: 1e-2, native.PRECISION_BF16X6: 1e-4}
PRECISIONS = [native.PRECISION_BF16X3, native.PRECISION_TF32, native.PRECISION_BF16X6]


@pytest.fixture(params=PRECISIONS, ids=["bf16x3", "tf32", "bf16x6"])
def reduced(request, gpu):
    old = native.set_precision(request.param)
    yield request.param
    native.set_precision(old)


@pytest.fixture(params=[64, 128, 256], ids=["bn64", "bn128", "bn256"])
def tile_width(request, gpu):
    """Force the tensor-core tile width (the autotuner would choose, possibly FP64 for small products)."""
    gpu.ctgpu_clear_plan_cache()
    assert gpu.ctgpu_set_tc_tile_width(request.param) == 0
    yield request.param
    gpu.ctgpu_set_tc_tile_width(0)
    gpu.ctgpu_clear_plan_cache()


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


def _random_pair(seed, shape):
    rng = np.random.default_rng(500 + seed)
    # "tiles": blocks larger than one tensor-core tile in both directions and K over several chunks
    lo, hi = (2, 14) if shape == "small" else (60, 300)
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
    return s, axs, t, axt


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("shape", ["small", "tiles"])
def test_reduced_dot_matches_oracle(reduced, tile_width, oracle_port, seed, shape):
    s, axs, t, axt = _random_pair(seed, shape)
    got = _dot(native.lib().ctgpu_block_sparse_tensor_dot, s, axs, t, axt, 1)
    ref = _dot(oracle_port.oracle_block_sparse_tensor_dot, s, axs, t, axt, 1, check=False)
    bound = _dot(oracle_port.oracle_block_sparse_tensor_dot, _abs_bst(s), axs, _abs_bst(t), axt, 1, check=False)
    assert got.dim_logical == ref.dim_logical and set(got.blocks) == set(ref.blocks)
    tol = DOT_RTOL[reduced]
    for k, v in ref.blocks.items():
        assert np.all(np.abs(got.blocks[k] - v) <= tol * bound.blocks[k] + 1e-300), k


def test_three_part_split_is_more_accurate(tile_width, oracle_port):
    """With a short contraction (k = 16: one accumulator update per product) the six-product form
    is far closer to FP64 than the three-product one: its operands keep 24 bits instead of 16. On
    long contractions both are limited by the FP32 accumulation on the tensor cores instead."""
    gpu = native.lib()
    rng = np.random.default_rng(77)
    z = lambda n: np.zeros(n, np.int32)
    s = cs.BlockSparse((200, 16), (1, 1), [z(200), z(16)])
    t = cs.BlockSparse((16, 150), (-1, 1), [z(16), z(150)])
    s.blocks[(0, 0)] = rng.standard_normal((200, 16))
    t.blocks[(0, 0)] = rng.standard_normal((16, 150))
    ref = s.blocks[(0, 0)] @ t.blocks[(0, 0)]
    bound = np.abs(s.blocks[(0, 0)]) @ np.abs(t.blocks[(0, 0)])
    err = {}
    for p in (native.PRECISION_BF16X3, native.PRECISION_BF16X6):
        old = native.set_precision(p)
        try:
            got = _dot(gpu.ctgpu_block_sparse_tensor_dot, s, 1, t, 0, 1)
        finally:
            native.set_precision(old)
        err[p] = float((np.abs(got.blocks[(0, 0)] - ref) / bound).max())
    assert err[native.PRECISION_BF16X6] * 10 < err[native.PRECISION_BF16X3], err
    assert err[native.PRECISION_BF16X6] < 1e-6, err


def test_reduced_local_hamiltonian_matches_reference(reduced, tile_width):
    g = golden("local_ops_hubbard_L8.npz")
    t = {k: cs.bst_from_arrays(k, g) for k in ["h2", "l", "r", "a", "b"]}
    c = {k: c_bst(v) for k, v in t.items()}
    out = cs.BlockSparseTensor()
    assert native.lib().ctgpu_apply_local_hamiltonian(C.byref(c["a"]), C.byref(c["h2"]), C.byref(c["l"]),
                                                      C.byref(c["r"]), C.byref(out)) == 0
    got = cs.read_bst(out)
    cs.free_bst(out)
    num = sum(float(np.sum((got.blocks[k] - v) ** 2)) for k, v in t["b"].blocks.items())
    den = sum(float(np.sum(v ** 2)) for v in t["b"].blocks.values())
    assert np.sqrt(num / den) < LOCAL_H_RTOL[reduced]
    for v in c.values():
        cs.free_bst(v)


def test_reduced_dmrg_final_fp64_sweep(reduced, oracle_port):
    """Reduced-precision sweeps followed by one FP64 sweep land on the converged FP64 energy:
    to 1e-8 for the split-BF16 forms, to 1e-6 for TF32. The tile width is forced, so that every
    product runs on the tensor cores (the autotuner would keep this small problem on FP64)."""
    gpu = native.lib()
    gpu.ctgpu_clear_plan_cache()
    assert gpu.ctgpu_set_tc_tile_width(128) == 0
    H = hm.fermi_hubbard_1d(12, 1.0, 4.0, 0.0)
    c = native.random_mps(12, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(12, 0), 48, 11)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    old = gpu.ctgpu_set_profiling(1, 0)
    try:
        r1, e1, s1, p1 = run_gpu_dmrg(gpu, H, psi0, 8, 5, 1e-10, 48)
    finally:
        gpu.ctgpu_set_profiling(old, 0)
        gpu.ctgpu_set_tc_tile_width(0)
        gpu.ctgpu_clear_plan_cache()
    assert r1 == 0, native.last_error()
    prof = native.kernel_profile()
    # the tensor-core kernel ran in the reduced sweeps and the FP64 kernel in the final one
    assert prof["block_gemm_tc"]["launches"] > 0 and prof["block_gemm"]["launches"] > 0
    r2, e2, s2, p2 = run_oracle_dmrg(oracle_port, H, psi0, 8, 5, 1e-10, 48)
    assert r2 == 0
    # the reduced sweeps agree with FP64 to the format's accuracy (the energy of a reduced-precision
    # local Hamiltonian is not variational and may fall slightly below the FP64 value) ...
    sweep_rtol = {native.PRECISION_BF16X3: 5e-4, native.PRECISION_TF32: 2e-2, native.PRECISION_BF16X6: 5e-4}[reduced]
    np.testing.assert_allclose(e1[:-1], e2[:-1], rtol=sweep_rtol, atol=0)
    # ... and the final FP64 sweep reaches the FP64 energy
    assert abs(e1[-1] - e2[-1]) <= (1e-6 if reduced == native.PRECISION_TF32 else 1e-8)
    assert native.last_stats()["matvecs"] > 0


def test_tile_autotuner_records_its_choices(gpu):
    """With no forced width, planning a tensor-core product times the three widths once per
    work-list histogram and reports the pick."""
    gpu.ctgpu_set_tc_tile_width(0)
    gpu.ctgpu_clear_plan_cache()
    old = native.set_precision(native.PRECISION_BF16X3)
    try:
        s, axs, t, axt = _random_pair(3, "tiles")
        _dot(gpu.ctgpu_block_sparse_tensor_dot, s, axs, t, axt, 1)
    finally:
        native.set_precision(old)
    entries = native.tile_tuning()
    assert entries and all(e["bn"] in (0, 64, 128, 256) for e in entries)
    assert any(e["key"].startswith("p1_") for e in entries)


def test_set_precision_rejects_unknown_values(gpu):
    assert native.lib().ctgpu_set_precision(7) < 0
    assert native.lib().ctgpu_set_tc_tile_width(96) < 0
    old = native.set_precision(native.PRECISION_FP64)
    assert native.set_precision(old) == native.PRECISION_FP64
