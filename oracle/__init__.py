"""CPU oracle for the two-site DMRG path. TEST INFRASTRUCTURE ONLY.

Loads the C restatement (ct_oracle.c, built by ``make -C oracle port``) and,
where it was built, the reference compiled from its own sources
(oracle/_ref/libct_ref.so). Only the tests, the smoke check and the CPU
baseline leg of bench.py use this package; the product never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PORT = os.path.join(HERE, "_build", "liboracle.so")
REF = os.path.join(HERE, "_ref", "libct_ref.so")


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT


def build_ref(refdir: str | None = None) -> str | None:
    """Compile the reference from its own sources into _ref/ (x86 container only). The checkout is
    named by the argument or the CHEMTENSOR_REFERENCE_DIR environment variable; None if absent."""
    refdir = refdir or os.environ.get("CHEMTENSOR_REFERENCE_DIR")
    if not refdir or not os.path.isdir(refdir):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFDIR={refdir}"], check=True)
    return REF


_port = None


def port() -> C.CDLL:
    """The C restatement; built on first use."""
    global _port
    if _port is None:
        os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
        if not os.path.exists(PORT):
            build_port()
        lib = C.CDLL(PORT)
        P = C.c_void_p
        lib.oracle_dmrg_twosite.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_int64, P, P, P]
        lib.oracle_dmrg_singlesite.argtypes = [P, C.c_int, C.c_int, P, P]
        lib.oracle_apply_local_hamiltonian.argtypes = [P] * 5
        lib.oracle_block_sparse_tensor_qr.argtypes = [P, P, P]
        lib.oracle_block_sparse_tensor_rq.argtypes = [P, P, P]
        lib.oracle_block_sparse_tensor_dot.argtypes = [P, C.c_int, P, C.c_int, C.c_int, P]
        lib.oracle_block_sparse_tensor_transpose.argtypes = [P, P, P]
        lib.oracle_block_sparse_tensor_svd.argtypes = [P, P, P, P, P]
        lib.oracle_contraction_operator_step_left.argtypes = [P] * 5
        lib.oracle_contraction_operator_step_right.argtypes = [P] * 5
        lib.oracle_mps_vdot.argtypes = [P, P]
        lib.oracle_mps_vdot.restype = C.c_double
        lib.oracle_retained_bond_indices.argtypes = [P, C.c_int64, C.c_double, C.c_int, C.c_int64, P, P, P, P]
        lib.oracle_retained_bond_indices.restype = C.c_int64
        lib.oracle_lanczos_dense.argtypes = [C.c_int64, P, P, C.c_int, P, P]
        lib.oracle_delete_block_sparse_tensor.argtypes = [P]
        lib.oracle_delete_block_sparse_tensor.restype = None
        lib.oracle_set_num_threads.argtypes = [C.c_int]
        lib.oracle_get_sweep_times.argtypes = [P, C.c_int]
        lib.oracle_get_bond_sigma.argtypes = [C.c_int, P, C.c_int64]
        lib.oracle_get_bond_sigma.restype = C.c_int64
        lib.oracle_construct_random_mps.argtypes = [C.c_int, C.c_int64, P, C.c_int32, C.c_int64, C.c_uint64, P]
        _port = lib
    return _port


def reference() -> C.CDLL | None:
    """The reference itself (compiled here from its sources), or None where absent."""
    if not os.path.exists(REF):
        return None
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    lib = C.CDLL(REF)
    P = C.c_void_p
    lib.dmrg_twosite.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_int64, P, P, P]
    lib.ref_mps_vdot_real.argtypes = [P, P]
    lib.ref_mps_vdot_real.restype = C.c_double
    return lib


def bond_sigma(lib: C.CDLL, bond: int):
    """Retained singular values of the last split at `bond` in the last oracle_dmrg_twosite call."""
    import numpy as np
    n = lib.oracle_get_bond_sigma(bond, None, 0)
    if n < 0:
        return None
    out = np.zeros(max(n, 1))
    lib.oracle_get_bond_sigma(bond, out.ctypes.data, n)
    return out[:n]
