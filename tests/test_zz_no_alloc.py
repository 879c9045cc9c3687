"""The allocation-free dense SVD entry point (ctgpu_dense_svd_noalloc).

It serves callers that must not allocate device memory while they run, such as a service whose
device memory is reserved up front by its own pool, or code whose stream must not be stalled by
the implicit device-wide synchronisation of cudaMalloc / cudaFree. Its workspace is a fixed array
inside the library, so it only takes blocks of up to 256 x 256.

This file is collected last so that a run stopping at the first failure has already run every
other test. Device buffers come from torch (plumbing only); the SVD runs in libctgpu.so.
"""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs
from helpers import c_bst

pytestmark = pytest.mark.gpu

MAX_DIM = 256


def _graded(rng, m, n):
    u, _ = np.linalg.qr(rng.standard_normal((m, m)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    k = min(m, n)
    return (u[:, :k] * np.logspace(0, -9, k)) @ v[:, :k].T


def _svd_values_existing(gpu, a):
    """Singular values from the existing entry point, on a one-block block-sparse matrix."""
    m, n = a.shape
    t = cs.BlockSparse((m, n), (1, -1), [np.zeros(m, dtype=np.int32), np.zeros(n, dtype=np.int32)])
    t.blocks[(0, 0)] = a
    ct = c_bst(t)
    sig = np.zeros(min(m, n))
    ns = C.c_int64()
    assert gpu.ctgpu_block_sparse_tensor_svd_values(C.byref(ct), sig.ctypes.data, C.byref(ns)) == 0
    cs.free_bst(ct)
    return sig[:ns.value]


def test_dense_svd_noalloc_matches_block_svd(gpu):
    torch = pytest.importorskip("torch")
    fn = gpu.ctgpu_dense_svd_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(2024)
    # two calls in a row share the library's fixed workspace; the second must not see the first
    for m, n in [(200, 150), (96, 230)]:
        a = _graded(rng, m, n)
        k = min(m, n)
        d_a = torch.from_numpy(a).to(dev)
        d_u = torch.full((m * k,), np.nan, dtype=torch.float64, device=dev)
        d_s = torch.full((k,), np.nan, dtype=torch.float64, device=dev)
        d_vh = torch.full((k * n,), np.nan, dtype=torch.float64, device=dev)
        d_info = torch.full((1,), 7, dtype=torch.int32, device=dev)
        ret = fn(d_a.data_ptr(), m, n, d_u.data_ptr(), d_s.data_ptr(), d_vh.data_ptr(), d_info.data_ptr(),
                 stream.cuda_stream)
        assert ret == 0
        torch.cuda.synchronize(dev)
        assert int(d_info.item()) == 0
        s = d_s.cpu().numpy()
        u = d_u.cpu().numpy().reshape(m, k)
        vh = d_vh.cpu().numpy().reshape(k, n)
        ref = _svd_values_existing(gpu, a)
        # same tolerances as the other block SVD tests
        np.testing.assert_allclose(s, ref, rtol=1e-10, atol=1e-14 * ref.max())
        assert np.all(np.diff(s) <= 0)
        np.testing.assert_allclose((u * s) @ vh, a, rtol=0, atol=1e-12 * np.abs(a).max())
        np.testing.assert_allclose(u.T @ u, np.eye(k), rtol=0, atol=1e-10)
        np.testing.assert_allclose(vh @ vh.T, np.eye(k), rtol=0, atol=1e-10)


@pytest.mark.parametrize("m,n", [(1, 1), (1, 7), (7, 1), (3, 2), (256, 256), (256, 17), (17, 256)])
def test_dense_svd_noalloc_edge_shapes(gpu, m, n):
    """The documented limits: single rows and columns, tiny blocks (most CTAs of the cluster own no
    column) and the 256 x 256 maximum the fixed workspace is sized for."""
    torch = pytest.importorskip("torch")
    fn = gpu.ctgpu_dense_svd_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(m * 1000 + n)
    a = _graded(rng, m, n) if min(m, n) > 1 else rng.standard_normal((m, n))
    k = min(m, n)
    d_a = torch.from_numpy(a).to(dev)
    d_u = torch.full((m * k,), np.nan, dtype=torch.float64, device=dev)
    d_s = torch.full((k,), np.nan, dtype=torch.float64, device=dev)
    d_vh = torch.full((k * n,), np.nan, dtype=torch.float64, device=dev)
    d_info = torch.full((1,), 7, dtype=torch.int32, device=dev)
    assert fn(d_a.data_ptr(), m, n, d_u.data_ptr(), d_s.data_ptr(), d_vh.data_ptr(), d_info.data_ptr(),
              stream.cuda_stream) == 0
    torch.cuda.synchronize(dev)
    assert int(d_info.item()) == 0
    s = d_s.cpu().numpy()
    u = d_u.cpu().numpy().reshape(m, k)
    vh = d_vh.cpu().numpy().reshape(k, n)
    ref = np.linalg.svd(a, compute_uv=False)
    np.testing.assert_allclose(s, ref, rtol=1e-10, atol=1e-14 * ref.max())
    assert np.all(np.diff(s) <= 0)
    np.testing.assert_allclose((u * s) @ vh, a, rtol=0, atol=1e-12 * np.abs(a).max())
    np.testing.assert_allclose(u.T @ u, np.eye(k), rtol=0, atol=1e-10)
    np.testing.assert_allclose(vh @ vh.T, np.eye(k), rtol=0, atol=1e-10)


def test_dense_svd_noalloc_rejects_oversized_blocks(gpu):
    torch = pytest.importorskip("torch")
    fn = gpu.ctgpu_dense_svd_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    dev = torch.device("cuda:0")
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    p = buf.data_ptr()
    assert fn(p, MAX_DIM + 1, 4, p, p, p, info.data_ptr(), None) == -5
    assert fn(p, 4, 0, p, p, p, info.data_ptr(), None) == -5
