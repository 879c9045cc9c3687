"""Shared helpers of the test suite: C-struct round trips and gauge-invariant comparisons."""

import ctypes as C

import numpy as np

from chemtensor_gb300 import ctstructs as cs


def c_bst(t: cs.BlockSparse) -> cs.BlockSparseTensor:
    c = cs.BlockSparseTensor()
    cs.write_bst(t, c)
    return c


def run_oracle_dmrg(port, H: cs.Chain, psi0: cs.Chain, sweeps, maxiter, tol, D):
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en = np.zeros(sweeps)
    ent = np.zeros(H.nsites - 1)
    ret = port.oracle_dmrg_twosite(C.byref(cH), sweeps, maxiter, tol, D, C.byref(cP), en.ctypes.data, ent.ctypes.data)
    out = cs.read_mps(cP)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    return ret, en, ent, out


def run_gpu_dmrg(lib, H: cs.Chain, psi0: cs.Chain, sweeps, maxiter, tol, D):
    cH, cP = cs.make_c_mpo(H), cs.make_c_mps(psi0)
    en = np.zeros(sweeps)
    ent = np.zeros(H.nsites - 1)
    ret = lib.dmrg_twosite(C.byref(cH), sweeps, maxiter, tol, D, C.byref(cP), en.ctypes.data, ent.ctypes.data)
    out = cs.read_mps(cP)
    cs.free_mps(cP)
    cs.free_mpo(cH)
    return ret, en, ent, out


def overlap(port, a: cs.Chain, b: cs.Chain) -> float:
    ca, cb = cs.make_c_mps(a), cs.make_c_mps(b)
    v = port.oracle_mps_vdot(C.byref(ca), C.byref(cb))
    cs.free_mps(ca)
    cs.free_mps(cb)
    return v


def same_structure(a: cs.Chain, b: cs.Chain) -> bool:
    if a.nsites != b.nsites:
        return False
    for x, y in zip(a.tensors, b.tensors):
        if x.dim_logical != y.dim_logical or x.axis_dir != y.axis_dir:
            return False
        if not all(np.array_equal(p, q) for p, q in zip(x.qnums_logical, y.qnums_logical)):
            return False
    return True


def assert_bst_close(x: cs.BlockSparse, y: cs.BlockSparse, rtol: float):
    assert x.dim_logical == y.dim_logical and x.axis_dir == y.axis_dir
    for p, q in zip(x.qnums_logical, y.qnums_logical):
        assert np.array_equal(p, q)
    assert x.allowed == y.allowed
    u, v = x.serialize(), y.serialize()
    scale = max(np.abs(v).max(initial=0.0), 1e-300)
    assert np.abs(u - v).max(initial=0.0) <= rtol * scale, np.abs(u - v).max() / scale
