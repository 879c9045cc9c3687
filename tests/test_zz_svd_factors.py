"""Block SVD factors at the ranks where the Jacobi sweeps start from an FP32-preconditioned basis
(rank 48 and up): singular values against LAPACK (numpy), orthonormal factors and the
reconstruction, for graded, numerically rank-deficient and clustered spectra like those of the
two-site DMRG bond matrices.

The dense allocation-free entry point (ctgpu_dense_svd_noalloc) runs the same cluster kernel as
the block SVD of the DMRG path and returns all three factors. Collected after the other GPU tests
(device buffers come from torch, as plumbing only).
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spectrum(rng, m, n, kind):
    k = min(m, n)
    u, _ = np.linalg.qr(rng.standard_normal((m, m)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    if kind == "graded":
        s = np.logspace(0, -9, k)
    elif kind == "lowrank":
        # exact rank 60 plus rounding-level noise
        s = np.concatenate([np.logspace(0, -12, 60), np.zeros(k - 60)])
    else:
        # clusters of (nearly) equal values: degenerate subspaces
        s = np.repeat(np.logspace(0, -6, (k + 3) // 4), 4)[:k] * (1 + 1e-13 * np.arange(k))
    a = (u[:, :k] * s) @ v[:, :k].T
    if kind == "lowrank":
        a += 1e-16 * rng.standard_normal((m, n))
    return a


@pytest.mark.parametrize("m,n,kind", [
    (120, 100, "graded"), (100, 120, "graded"), (136, 136, "graded"), (64, 200, "graded"),
    (128, 96, "lowrank"), (112, 112, "clustered"), (60, 50, "graded"),
])
def test_svd_factors_preconditioned_ranks(gpu, m, n, kind):
    torch = pytest.importorskip("torch")
    fn = gpu.ctgpu_dense_svd_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(m * 1000 + n)
    a = _spectrum(rng, m, n, kind)
    k = min(m, n)
    d_a = torch.from_numpy(a).to(dev)
    d_u = torch.zeros((m * k,), dtype=torch.float64, device=dev)
    d_s = torch.zeros((k,), dtype=torch.float64, device=dev)
    d_vh = torch.zeros((k * n,), dtype=torch.float64, device=dev)
    d_info = torch.full((1,), 7, dtype=torch.int32, device=dev)
    assert fn(d_a.data_ptr(), m, n, d_u.data_ptr(), d_s.data_ptr(), d_vh.data_ptr(), d_info.data_ptr(),
              stream.cuda_stream) == 0
    torch.cuda.synchronize(dev)
    assert int(d_info.item()) == 0
    s = d_s.cpu().numpy()
    u = d_u.cpu().numpy().reshape(m, k)
    vh = d_vh.cpu().numpy().reshape(k, n)
    ref = np.linalg.svd(a, compute_uv=False)
    big = ref > 1e-6 * ref[0]
    # retained singular values (DMRG keeps values above ~1e-5 sigma_max; bar 1e-8 relative)
    np.testing.assert_allclose(s[big], ref[big], rtol=1e-10)
    # the rest at LAPACK's own absolute accuracy (~(m + n) eps sigma_max)
    np.testing.assert_allclose(s, ref, rtol=0, atol=2e-12 * ref[0])
    assert np.all(np.diff(s) <= 0)
    np.testing.assert_allclose((u * s) @ vh, a, rtol=0, atol=1e-12 * np.abs(a).max())
    # factors orthonormal to FP64 rounding over the numerically nonzero directions
    r = int(np.sum(s > 1e-13 * s[0]))
    np.testing.assert_allclose(u[:, :r].T @ u[:, :r], np.eye(r), rtol=0, atol=1e-12)
    np.testing.assert_allclose(vh[:r] @ vh[:r].T, np.eye(r), rtol=0, atol=1e-12)


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("m,n,kind", [
    (112, 112, "clustered"), (128, 120, "graded"), (150, 140, "clustered"), (100, 96, "clustered"),
    (140, 150, "graded"),
])
def test_svd_factors_seeded_spectra(gpu, seed, m, n, kind):
    """More seeds of the graded and four-fold clustered spectra (the refinement finish, its exact
    cluster rotations and the FP64 sweeps it hands over to): orthonormal factors, reconstruction
    and the retained singular values at the same bars."""
    torch = pytest.importorskip("torch")
    fn = gpu.ctgpu_dense_svd_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(seed * 7919 + m * 1000 + n)
    a = _spectrum(rng, m, n, kind)
    k = min(m, n)
    d_a = torch.from_numpy(a).to(dev)
    d_u = torch.zeros((m * k,), dtype=torch.float64, device=dev)
    d_s = torch.zeros((k,), dtype=torch.float64, device=dev)
    d_vh = torch.zeros((k * n,), dtype=torch.float64, device=dev)
    d_info = torch.full((1,), 7, dtype=torch.int32, device=dev)
    assert fn(d_a.data_ptr(), m, n, d_u.data_ptr(), d_s.data_ptr(), d_vh.data_ptr(), d_info.data_ptr(),
              stream.cuda_stream) == 0
    torch.cuda.synchronize(dev)
    assert int(d_info.item()) == 0
    s = d_s.cpu().numpy()
    u = d_u.cpu().numpy().reshape(m, k)
    vh = d_vh.cpu().numpy().reshape(k, n)
    ref = np.linalg.svd(a, compute_uv=False)
    big = ref > 1e-6 * ref[0]
    np.testing.assert_allclose(s[big], ref[big], rtol=1e-10)
    np.testing.assert_allclose((u * s) @ vh, a, rtol=0, atol=1e-12 * np.abs(a).max())
    r = int(np.sum(s > 1e-13 * s[0]))
    np.testing.assert_allclose(u[:, :r].T @ u[:, :r], np.eye(r), rtol=0, atol=1e-12)
    np.testing.assert_allclose(vh[:r] @ vh[:r].T, np.eye(r), rtol=0, atol=1e-12)
