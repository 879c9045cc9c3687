"""Error paths of the GPU implementation, made on the host (no GPU fault is provoked).

The reference's failure codes (src/util/krylov.c:218-236, src/tensor/block_sparse_tensor.c:
2843-2847, propagated by src/algorithm/dmrg.c:312-355) reach the caller of dmrg_twosite:
  -1  a start vector of norm zero (the host zeroes it; the device's norm check stops the Lanczos
      iteration before its first eigenvalue), or a block SVD that did not converge (injected on the
      host: the SVD's status word is read back normally and then overridden);
  -2  a failed tridiagonal eigensolve (injected on the host the same way);
  -5  a tensor-core GEMM whose bounded mbarrier waits ran out: the limit is lowered to one poll, so
      the kernel takes its own error exit (records a flag, lets its copies land, frees its tensor
      memory and returns) and the call reports it; the context stays usable.
"""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm, native
from helpers import c_bst, run_gpu_dmrg

pytestmark = pytest.mark.gpu


def _hubbard(L=8, D=24, seed=5):
    H = hm.fermi_hubbard_1d(L, 1.0, 4.0, 0.0)
    c = native.random_mps(L, 4, hm.HUBBARD_QSITE, hm.encode_quantum_number_pair(L, 0), D, seed)
    psi0 = cs.read_mps(c)
    cs.free_mps(c)
    return H, psi0


def test_zero_start_vector_returns_minus_one(gpu):
    """A local eigenproblem whose start vector is zero (zeroed by the host) ends in the Lanczos
    breakdown exit. (A zero input MPS does not get there: its right normalisation leaves
    isometries, as in the reference.)"""
    H, psi0 = _hubbard()
    assert gpu.ctgpu_inject_failure(3, 1) == 0
    try:
        ret, *_ = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 24)
    finally:
        gpu.ctgpu_inject_failure(3, 0)
    assert ret == -1


def test_injected_svd_failure_returns_minus_one(gpu):
    H, psi0 = _hubbard()
    assert gpu.ctgpu_inject_failure(1, 1) == 0
    try:
        ret, *_ = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 24)
    finally:
        gpu.ctgpu_inject_failure(1, 0)
    assert ret == -1
    # the next call is unaffected
    ret, en, *_ = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 24)
    assert ret == 0 and np.all(np.isfinite(en))


def test_injected_tridiagonal_failure_returns_minus_two(gpu):
    H, psi0 = _hubbard()
    assert gpu.ctgpu_inject_failure(2, 1) == 0
    try:
        ret, *_ = run_gpu_dmrg(gpu, H, psi0, 2, 5, 1e-10, 24)
    finally:
        gpu.ctgpu_inject_failure(2, 0)
    assert ret == -2
    assert gpu.ctgpu_inject_failure(4, 1) == -5


def test_tensor_core_wait_limit_error_exit(gpu):
    """A bounded wait that runs out ends the tensor-core GEMM through its error exit: the call
    returns -5 with a message, and the same call succeeds once the limit is restored."""
    rng = np.random.default_rng(3)
    s = cs.BlockSparse((400, 300), (1, 1), [np.zeros(400, np.int32), np.zeros(300, np.int32)])
    t = cs.BlockSparse((300, 500), (-1, 1), [np.zeros(300, np.int32), np.zeros(500, np.int32)])
    s.blocks[(0, 0)] = rng.standard_normal((400, 300))
    t.blocks[(0, 0)] = rng.standard_normal((300, 500))
    cs_, ct_ = c_bst(s), c_bst(t)
    old = native.set_precision(native.PRECISION_BF16X3)
    try:
        gpu.ctgpu_set_tc_wait_limit(1)
        out = cs.BlockSparseTensor()
        ret = gpu.ctgpu_block_sparse_tensor_dot(C.byref(cs_), 1, C.byref(ct_), 0, 1, C.byref(out))
        msg = native.last_error()
        if ret == 0:
            cs.free_bst(out)
        gpu.ctgpu_set_tc_wait_limit(0)
        assert ret == -5 and "timed out" in msg, (ret, msg)
        out = cs.BlockSparseTensor()
        assert gpu.ctgpu_block_sparse_tensor_dot(C.byref(cs_), 1, C.byref(ct_), 0, 1, C.byref(out)) == 0
        got = cs.read_bst(out)
        cs.free_bst(out)
        ref = s.blocks[(0, 0)] @ t.blocks[(0, 0)]
        assert np.abs(got.blocks[(0, 0)] - ref).max() <= 1e-3 * np.abs(ref).max()
    finally:
        gpu.ctgpu_set_tc_wait_limit(0)
        native.set_precision(old)
        cs.free_bst(cs_)
        cs.free_bst(ct_)
