"""complex128 (CT_DOUBLE_COMPLEX) on the GPU: two-site and single-site DMRG against the reference's
own complex runs, and the complex block operations (dot, QR / RQ, SVD) against numpy."""

import ctypes as C

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs
from conftest import golden
from helpers import c_bst, same_structure

pytestmark = pytest.mark.gpu


def mps_vector(ch: cs.Chain) -> np.ndarray:
    v = ch.tensors[0].to_dense()
    v = v.reshape(-1, v.shape[-1])
    for t in ch.tensors[1:]:
        a = t.to_dense()
        v = np.tensordot(v, a, axes=(1, 0)).reshape(-1, a.shape[-1])
    return v.ravel()


def _run(gpu, g, single):
    L, D, sweeps, maxiter = [int(x) for x in g["params"]]
    H = cs.chain_from_arrays("H", g)
    psi0 = cs.chain_from_arrays("psi0", g)
    assert H.tensors[0].dtype == cs.CT_DOUBLE_COMPLEX and psi0.tensors[0].dtype == cs.CT_DOUBLE_COMPLEX
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en, ent = np.zeros(sweeps), np.zeros(L - 1)
    if single:
        ret = gpu.dmrg_singlesite(C.byref(cH), sweeps, maxiter, C.byref(cP), en.ctypes.data)
    else:
        ret = gpu.dmrg_twosite(C.byref(cH), sweeps, maxiter, float(g["tol_split"]), D, C.byref(cP), en.ctypes.data,
                               ent.ctypes.data)
    psi = cs.read_mps(cP)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    return ret, en, ent, psi


@pytest.mark.parametrize("case,single", [("dmrg_complex_hubbard_L6_D32.npz", False),
                                         ("dmrg1_complex_hubbard_L6_D24.npz", True)])
def test_complex_dmrg_matches_reference(gpu, case, single):
    g = golden(case)
    ret, en, ent, psi = _run(gpu, g, single)
    assert ret == 0
    np.testing.assert_allclose(en, g["en_sweeps"], rtol=0, atol=1e-10)
    if not single:
        np.testing.assert_allclose(ent, g["entropy"], rtol=0, atol=1e-8)
    ref = cs.chain_from_arrays("psi", g)
    assert psi.tensors[0].dtype == cs.CT_DOUBLE_COMPLEX
    assert same_structure(psi, ref)
    u, v = mps_vector(psi), mps_vector(ref)
    assert abs(np.linalg.norm(u) - 1) < 1e-12
    assert abs(abs(np.vdot(v, u)) - 1) < 1e-9


def _random_complex(rng, dims, dirs, qrange):
    qn = [rng.integers(-qrange, qrange + 1, size=d).astype(np.int32) for d in dims]
    t = cs.BlockSparse(dims, dirs, qn, dtype=cs.CT_DOUBLE_COMPLEX)
    for idx in t.allowed:
        shp = t.block_shape(idx)
        t.blocks[idx] = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
    return t


@pytest.mark.parametrize("seed", range(3))
def test_complex_dot_matches_numpy(gpu, seed):
    rng = np.random.default_rng(500 + seed)
    s = _random_complex(rng, (7, 5, 9), (1, 1, -1), 2)
    qk = s.qnums_logical[2]
    t = cs.BlockSparse((9, 4, 6), (1, 1, -1), [qk, rng.integers(-2, 3, 4).astype(np.int32),
                                                 rng.integers(-3, 4, 6).astype(np.int32)], dtype=cs.CT_DOUBLE_COMPLEX)
    for idx in t.allowed:
        shp = t.block_shape(idx)
        t.blocks[idx] = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
    cs_, ct_ = c_bst(s), c_bst(t)
    out = cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_dot(C.byref(cs_), 1, C.byref(ct_), 0, 1, C.byref(out)) == 0
    got = cs.read_bst(out).to_dense()
    ref = np.tensordot(s.to_dense(), t.to_dense(), axes=(2, 0))
    assert np.abs(got - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.0)
    cs.free_bst(out)
    cs.free_bst(cs_)
    cs.free_bst(ct_)


@pytest.mark.parametrize("shape", [(30, 20), (20, 30), (16, 16)])
def test_complex_qr_rq_and_svd(gpu, shape):
    rng = np.random.default_rng(sum(shape))
    a = _random_complex(rng, shape, (1, -1), 2)
    ca = c_bst(a)
    A = a.to_dense()
    q, r = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_qr(C.byref(ca), 0, C.byref(q), C.byref(r)) == 0
    Q, R = cs.read_bst(q).to_dense(), cs.read_bst(r).to_dense()
    assert np.abs(Q @ R - A).max() <= 1e-12 * np.abs(A).max()
    assert np.abs(Q.conj().T @ Q - np.eye(Q.shape[1])).max() <= 1e-12
    r2, q2 = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    assert gpu.ctgpu_block_sparse_tensor_rq(C.byref(ca), 0, C.byref(r2), C.byref(q2)) == 0
    Q2, R2 = cs.read_bst(q2).to_dense(), cs.read_bst(r2).to_dense()
    assert np.abs(R2 @ Q2 - A).max() <= 1e-12 * np.abs(A).max()
    assert np.abs(Q2 @ Q2.conj().T - np.eye(Q2.shape[0])).max() <= 1e-12
    sig = np.zeros(min(shape))
    ns = C.c_int64()
    assert gpu.ctgpu_block_sparse_tensor_svd_values(C.byref(ca), sig.ctypes.data, C.byref(ns)) == 0
    ref = np.sort(np.concatenate([np.linalg.svd(b, compute_uv=False) for b in a.blocks.values()]))[::-1]
    np.testing.assert_allclose(np.sort(sig[:ns.value])[::-1][:len(ref)], ref, rtol=1e-11, atol=1e-13)
    for x in (q, r, r2, q2):
        cs.free_bst(x)
    cs.free_bst(ca)


def test_complex_mps_vdot_and_norm(gpu):
    g = golden("dmrg_complex_hubbard_L6_D32.npz")
    a, b = cs.chain_from_arrays("psi0", g), cs.chain_from_arrays("psi", g)
    ca, cb = cs.make_c_mps(a), cs.make_c_mps(b)
    va, vb = mps_vector(a), mps_vector(b)
    for x, y, ref in ((ca, cb, np.vdot(va, vb)), (cb, ca, np.vdot(vb, va)), (ca, ca, np.vdot(va, va))):
        got = (C.c_double * 2)()
        assert gpu.ctgpu_mps_vdot(C.byref(x), C.byref(y), got) == 0
        assert abs(complex(got[0], got[1]) - ref) <= 1e-12 * max(1.0, abs(ref))
    nrm = C.c_double()
    assert gpu.ctgpu_mps_norm(C.byref(ca), C.byref(nrm)) == 0
    assert abs(nrm.value - np.linalg.norm(va)) <= 1e-12 * nrm.value
    cs.free_mps(ca)
    cs.free_mps(cb)
