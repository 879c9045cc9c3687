"""Single device operations through the C ABI against the reference goldens and the oracle."""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs
from conftest import golden
from helpers import assert_bst_close, c_bst

pytestmark = pytest.mark.gpu

# FP64 block GEMMs sum in a different order than OpenBLAS: agreement to rounding
RTOL = 1e-12


def _run(fn, *args):
    out = cs.BlockSparseTensor()
    ret = fn(*[C.byref(a) for a in args], C.byref(out))
    assert ret == 0
    r = cs.read_bst(out)
    cs.free_bst(out)
    return r


@pytest.mark.parametrize("case", ["local_ops_heisenberg_L12.npz", "local_ops_hubbard_L8.npz"])
def test_local_ops_match_reference(gpu, case):
    g = golden(case)
    t = {k: cs.bst_from_arrays(k, g) for k in ["h2", "l", "r", "a", "b", "lnext", "rnext", "A", "B", "W", "W1"]}
    c = {k: c_bst(v) for k, v in t.items()}
    assert_bst_close(_run(gpu.ctgpu_apply_local_hamiltonian, c["a"], c["h2"], c["l"], c["r"]), t["b"], RTOL)
    assert_bst_close(_run(gpu.ctgpu_contraction_operator_step_left, c["A"], c["W"], c["l"]), t["lnext"], RTOL)
    assert_bst_close(_run(gpu.ctgpu_contraction_operator_step_right, c["B"], c["W1"], c["r"]), t["rnext"], RTOL)
    for v in c.values():
        cs.free_bst(v)


def _random_bst(rng, dims, dirs, qrange):
    qn = [rng.integers(-qrange, qrange + 1, size=d).astype(np.int32) for d in dims]
    t = cs.BlockSparse(dims, dirs, qn)
    for idx in t.allowed:
        t.blocks[idx] = rng.standard_normal(t.block_shape(idx))
    return t


@pytest.mark.parametrize("seed", range(6))
def test_dot_matches_oracle(gpu, oracle_port, seed):
    rng = np.random.default_rng(100 + seed)
    nmult = 1 + seed % 3
    axs, axt = seed % 2, (seed // 2) % 2
    nfs, nft = 1 + seed % 2, 2 - seed % 2
    cdims = [int(x) for x in rng.integers(3, 12, size=nmult)]
    cq = [rng.integers(-2, 3, size=d).astype(np.int32) for d in cdims]
    cdir = [int(x) for x in rng.choice([-1, 1], size=nmult)]
    fs = [int(x) for x in rng.integers(2, 14, size=nfs)]
    ft = [int(x) for x in rng.integers(2, 14, size=nft)]
    fsq = [rng.integers(-3, 4, size=d).astype(np.int32) for d in fs]
    ftq = [rng.integers(-3, 4, size=d).astype(np.int32) for d in ft]
    fsd = [int(x) for x in rng.choice([-1, 1], size=nfs)]
    ftd = [int(x) for x in rng.choice([-1, 1], size=nft)]
    if axs == 0:
        s = cs.BlockSparse(cdims + fs, cdir + fsd, cq + fsq)
    else:
        s = cs.BlockSparse(fs + cdims, fsd + cdir, fsq + cq)
    tdir = [-d for d in cdir]
    if axt == 0:
        t = cs.BlockSparse(cdims + ft, tdir + ftd, cq + ftq)
    else:
        t = cs.BlockSparse(ft + cdims, ftd + tdir, ftq + cq)
    for x in (s, t):
        for idx in x.allowed:
            x.blocks[idx] = rng.standard_normal(x.block_shape(idx))
    cs_, ct_ = c_bst(s), c_bst(t)
    out = cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_dot(C.byref(cs_), axs, C.byref(ct_), axt, nmult, C.byref(out)) == 0
    ref = cs.BlockSparseTensor()
    oracle_port.oracle_block_sparse_tensor_dot(C.byref(cs_), axs, C.byref(ct_), axt, nmult, C.byref(ref))
    assert_bst_close(cs.read_bst(out), cs.read_bst(ref), RTOL)
    cs.free_bst(out)
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(ref))
    cs.free_bst(cs_)
    cs.free_bst(ct_)


@pytest.mark.parametrize("perm", [(1, 2, 0, 3, 4), (2, 0, 1, 3, 4), (0, 3, 1, 2), (0, 1, 4, 2, 3), (1, 3, 4, 2, 0),
                                  (3, 0, 1, 2), (4, 2, 0, 1, 3), (1, 2, 3, 0), (0, 1, 3, 2, 4, 5)])
def test_transpose_bitwise(gpu, oracle_port, perm):
    # every permutation used on the DMRG path (chain_ops.c, mpo.c)
    rng = np.random.default_rng(len(perm) * 10 + perm[0])
    nd = len(perm)
    dims = [int(x) for x in rng.integers(1, 7, size=nd)]
    dirs = [int(x) for x in rng.choice([-1, 1], size=nd)]
    t = _random_bst(rng, dims, dirs, 2)
    ct = c_bst(t)
    p = (C.c_int * nd)(*perm)
    out = cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_transpose(p, C.byref(ct), C.byref(out)) == 0
    ref = cs.BlockSparseTensor()
    oracle_port.oracle_block_sparse_tensor_transpose(p, C.byref(ct), C.byref(ref))
    assert_bst_close(cs.read_bst(out), cs.read_bst(ref), 0.0)
    cs.free_bst(out)
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(ref))
    cs.free_bst(ct)


@pytest.mark.parametrize("shape", [(40, 30), (30, 40), (96, 96), (7, 200)])
def test_svd_values_match_oracle(gpu, oracle_port, shape):
    rng = np.random.default_rng(sum(shape))
    q0 = rng.integers(-3, 4, size=shape[0]).astype(np.int32)
    q1 = rng.integers(-3, 4, size=shape[1]).astype(np.int32)
    a = cs.BlockSparse(shape, (1, -1), [q0, q1])
    for idx in a.allowed:
        b = rng.standard_normal(a.block_shape(idx))
        # graded spectrum down to 1e-9 relative, as in truncated DMRG bonds
        u, s, vh = np.linalg.svd(b, full_matrices=False)
        s = np.logspace(0, -9, len(s))
        a.blocks[idx] = (u * s) @ vh
    ca = c_bst(a)
    sig = np.zeros(min(shape))
    ns = C.c_int64()
    assert gpu.ctgpu_block_sparse_tensor_svd_values(C.byref(ca), sig.ctypes.data, C.byref(ns)) == 0
    u, vh = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    sp, nsr = C.POINTER(C.c_double)(), C.c_int64()
    assert oracle_port.oracle_block_sparse_tensor_svd(C.byref(ca), C.byref(u), C.byref(sp), C.byref(nsr), C.byref(vh)) == 0
    ref = np.ctypeslib.as_array(sp, shape=(nsr.value,)).copy()
    assert ns.value == nsr.value
    got = sig[:ns.value]
    # retained singular values within 1e-8 relative (the path's bar), here far tighter
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-14 * ref.max())
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(u))
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(vh))
    cs.free_bst(ca)


@pytest.mark.parametrize("rank,noise", [(30, 1e-17), (30, 1e-15), (60, 0.0), (110, 1e-16)])
def test_svd_values_rank_deficient_blocks(gpu, oracle_port, rank, noise):
    """Two-site DMRG matrices are numerically rank deficient: exact low rank plus rounding-level
    noise, several blocks of ~120 columns (the shape of the D=256 Hubbard bonds)."""
    rng = np.random.default_rng(rank)
    dims = (480, 500)
    q0 = np.repeat(np.arange(4, dtype=np.int32), 120)
    q1 = np.repeat(np.arange(4, dtype=np.int32), 125)
    a = cs.BlockSparse(dims, (1, -1), [q0, q1])
    for idx in a.allowed:
        m, n = a.block_shape(idx)
        u, _ = np.linalg.qr(rng.standard_normal((m, rank)))
        v, _ = np.linalg.qr(rng.standard_normal((n, rank)))
        s = np.logspace(0, -12, rank)
        a.blocks[idx] = (u * s) @ v.T + noise * rng.standard_normal((m, n))
    ca = c_bst(a)
    sig = np.zeros(min(dims))
    ns = C.c_int64()
    assert gpu.ctgpu_block_sparse_tensor_svd_values(C.byref(ca), sig.ctypes.data, C.byref(ns)) == 0
    u, vh = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    sp, nsr = C.POINTER(C.c_double)(), C.c_int64()
    assert oracle_port.oracle_block_sparse_tensor_svd(C.byref(ca), C.byref(u), C.byref(sp), C.byref(nsr), C.byref(vh)) == 0
    ref = np.ctypeslib.as_array(sp, shape=(nsr.value,)).copy()
    got = sig[:ns.value]
    # dgesvd (the oracle) resolves singular values to ~eps sigma_max absolute: compare those above
    # 1e-6 sigma_max relatively (retained values in DMRG lie above ~1e-5 sigma_max, bar 1e-8) and
    # all of them at the oracle's own absolute accuracy
    big = ref > 1e-6 * ref.max()
    np.testing.assert_allclose(got[big], ref[big], rtol=1e-9)
    # directions at the rounding floor are resolved to ~(m + n) eps sigma_max absolute
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-12 * ref.max())
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(u))
    oracle_port.oracle_delete_block_sparse_tensor(C.byref(vh))
    cs.free_bst(ca)


@pytest.mark.parametrize("tag", ["m0", "m1", "m2", "m3", "m4"])
def test_qr_rq_match_reference(gpu, tag):
    """Householder QR / RQ kernel against the reference's LAPACK factors (same sign conventions:
    the factors agree entry by entry, not only up to the gauge of the connecting axis)."""
    g = golden("qr_rq_blocks.npz")
    a = c_bst(cs.bst_from_arrays(tag, g))
    q, r = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_qr(C.byref(a), 0, C.byref(q), C.byref(r)) == 0
    assert_bst_close(cs.read_bst(q), cs.bst_from_arrays(tag + "_qr_q", g), 1e-12)
    assert_bst_close(cs.read_bst(r), cs.bst_from_arrays(tag + "_qr_r", g), 1e-12)
    r2, q2 = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_rq(C.byref(a), 0, C.byref(r2), C.byref(q2)) == 0
    assert_bst_close(cs.read_bst(r2), cs.bst_from_arrays(tag + "_rq_r", g), 1e-12)
    assert_bst_close(cs.read_bst(q2), cs.bst_from_arrays(tag + "_rq_q", g), 1e-12)
    for x in (q, r, r2, q2):
        cs.free_bst(x)
    # QR_COMPLETE is not provided: an error code, not a silent reduced factorisation
    q3, r3 = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_qr(C.byref(a), 1, C.byref(q3), C.byref(r3)) == -5
    cs.free_bst(a)


@pytest.mark.parametrize("case", ["dmrg_heisenberg_L20_D32.npz", "dmrg_hubbard_L12_D48.npz"])
def test_mps_vdot_and_norm_match_oracle(gpu, oracle_port, case):
    """Device mps_vdot / mps_norm against the oracle's mps_vdot (mps.c:314-370) on the reference's
    start and optimised states (different bond structures, same sector)."""
    g = golden(case)
    a, b = cs.chain_from_arrays("psi0", g), cs.chain_from_arrays("psi", g)
    ca, cb = cs.make_c_mps(a), cs.make_c_mps(b)
    for x, y in ((ca, cb), (cb, ca), (ca, ca), (cb, cb)):
        got = C.c_double()
        assert gpu.ctgpu_mps_vdot(C.byref(x), C.byref(y), C.byref(got)) == 0
        ref = oracle_port.oracle_mps_vdot(C.byref(x), C.byref(y))
        assert abs(got.value - ref) <= 1e-12 * max(1.0, abs(ref))
    nrm = C.c_double()
    assert gpu.ctgpu_mps_norm(C.byref(ca), C.byref(nrm)) == 0
    assert abs(nrm.value - np.sqrt(oracle_port.oracle_mps_vdot(C.byref(ca), C.byref(ca)))) <= 1e-12 * nrm.value
    cs.free_mps(ca)
    cs.free_mps(cb)
