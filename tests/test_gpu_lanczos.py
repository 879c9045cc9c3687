"""The device tridiagonal eigensolver of the Lanczos iteration against LAPACK.

The reference diagonalises the k x k Lanczos matrix with dsteqr (src/util/krylov.c:230) and keeps
the lowest eigenpair; the GPU path solves for that pair on one warp (FP32 Sturm multisection, FP64
Newton on the characteristic polynomial, eigenvector of the twisted factorisation from the leading
and trailing minors, or from the LDL^T pivots where the minors leave their range), fused into the
last Lanczos step.
Lowest eigenvalue within 1e-13 of ||T||, eigenvector within 1e-12 (up to the sign convention:
largest-magnitude component positive).
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lowest(gpu, a, b):
    k = len(a)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b if k > 1 else np.zeros(1), dtype=np.float64)
    lam = C.c_double()
    y = np.zeros(k)
    ret = gpu.ctgpu_tridiag_lowest(a.ctypes.data, b.ctypes.data, k, C.byref(lam), y.ctypes.data)
    return ret, lam.value, y


def _check(gpu, a, b):
    k = len(a)
    T = np.diag(a) + (np.diag(b, 1) + np.diag(b, -1) if k > 1 else 0)
    w, v = np.linalg.eigh(T)
    ret, lam, y = _lowest(gpu, a, b)
    assert ret == 0
    scale = max(np.abs(T).sum(axis=1).max(), 1e-300)
    assert abs(lam - w[0]) <= 1e-13 * scale, (lam, w[0])
    ref = v[:, 0] * np.sign(v[np.argmax(np.abs(v[:, 0])), 0])
    gap = (w[1] - w[0]) / scale if k > 1 else 1.0
    assert np.abs(y - ref).max() <= 1e-12 / min(1.0, gap * 1e3), (y, ref)
    assert abs(np.linalg.norm(y) - 1) < 1e-13


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 16, 25, 32])
@pytest.mark.parametrize("seed", range(3))
def test_tridiag_random(gpu, k, seed):
    rng = np.random.default_rng(100 * k + seed)
    scale = 10.0 ** rng.uniform(-3, 3)
    a = rng.standard_normal(k) * scale - 50.0 * scale * seed
    b = np.abs(rng.standard_normal(max(k - 1, 0))) * scale + 1e-3 * scale
    _check(gpu, a, b)


def test_tridiag_lanczos_like(gpu):
    """Converging Lanczos matrices: tiny trailing beta, the lowest Ritz value nearly exact."""
    for tail in (1e-3, 1e-6, 1e-9):
        a = np.array([-40.1, -39.7, -38.2, -35.0, -31.5])
        b = np.array([2.3, 1.1, 0.4, tail])
        _check(gpu, a, b)


def test_tridiag_eigenvector_concentrated_at_the_top(gpu):
    """A converging Lanczos run: the lowest Ritz vector lives in the leading components and is
    negligible at the end of the chain (a small beta decouples it), which a plain bottom-up
    recurrence cannot resolve."""
    a = np.array([-12.0, -3.5, 1.2, 2.5, 4.0])
    for tiny in (1e-4, 1e-7, 1e-10):
        _check(gpu, a, np.array([0.8, tiny, 0.6, 0.3]))
        _check(gpu, a[::-1].copy(), np.array([0.3, 0.6, tiny, 0.8]))


def test_tridiag_wilkinson(gpu):
    """Wilkinson's W21+ (pairs of nearly equal eigenvalues at the top of the spectrum)."""
    a = np.abs(np.arange(-10, 11)).astype(np.float64)
    b = np.ones(20)
    _check(gpu, a, b)


@pytest.mark.parametrize("scale", [1e7, 1e-7])
def test_tridiag_pivot_form_beyond_the_minor_range(gpu, scale):
    """Spreads whose leading minors leave [2^-600, 2^600] at k = 32: the solver takes its pivot form
    (LDL^T pivots) instead of the minors, with the same accuracy."""
    for seed in range(3):
        rng = np.random.default_rng(7000 + seed)
        a = rng.standard_normal(32) * scale
        b = np.abs(rng.standard_normal(31)) * scale + 1e-3 * scale
        _check(gpu, a, b)


def test_tridiag_rejects_bad_size(gpu):
    assert _lowest(gpu, np.zeros(33), np.ones(32))[0] == -5
