"""Loader and ctypes signatures of libctgpu.so (declared in include/ctgpu.h).

The library is built in-tree by ``chemtensor_gb300.build``. There is no
fallback: if the library is missing, importing this module raises.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ctstructs as cs

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libctgpu.so")

# exported C symbols (include/ctgpu.h)
EXPORTS = [
    "dmrg_twosite",
    "dmrg_singlesite",
    "ctgpu_set_precision",
    "ctgpu_set_reduced_environments",
    "ctgpu_set_device",
    "ctgpu_get_last_stats",
    "ctgpu_last_error",
    "ctgpu_construct_random_mps",
    "ctgpu_randn_sequence",
    "ctgpu_block_sparse_tensor_dot",
    "ctgpu_block_sparse_tensor_transpose",
    "ctgpu_apply_local_hamiltonian",
    "ctgpu_time_local_hamiltonian",
    "ctgpu_clear_plan_cache",
    "ctgpu_contraction_operator_step_left",
    "ctgpu_contraction_operator_step_right",
    "ctgpu_block_sparse_tensor_svd_values",
    "ctgpu_block_sparse_tensor_qr",
    "ctgpu_construct_spin_molecular_mpo",
    "ctgpu_mps_vdot",
    "ctgpu_device_memory",
    "ctgpu_mps_norm",
    "ctgpu_block_sparse_tensor_rq",
    "ctgpu_delete_block_sparse_tensor",
    "ctgpu_set_profiling",
    "ctgpu_set_l2_flush_bytes",
    "ctgpu_get_sweep_times",
    "ctgpu_get_kernel_profile",
    "ctgpu_measure_fp64_tflops",
    "ctgpu_get_bond_singular_values",
    "ctgpu_dense_svd_noalloc",
    "ctgpu_tile_tuning_report",
    "ctgpu_set_tc_tile_width",
    "ctgpu_set_tc_wait_limit",
    "ctgpu_inject_failure",
    "ctgpu_tridiag_lowest",
    "ctgpu_mpo_inner_product",
    "ctgpu_set_final_fp64_sweeps",
]

KERNEL_CLASSES = ["block_gemm", "permute", "row_map", "axis_scale", "block_svd", "block_rq", "lanczos_vector",
                  "block_gemm_tc"]

# arithmetic of the bulk block GEMMs (ctgpu_set_precision)
PRECISION_FP64 = 0
PRECISION_BF16X3 = 1
PRECISION_TF32 = 2
PRECISION_BF16X6 = 3
PRECISION_NAMES = {"fp64": 0, "bf16x3": 1, "tf32": 2, "bf16x6": 3}


class Stats(C.Structure):
    _fields_ = [
        ("wall_s", C.c_double), ("upload_s", C.c_double), ("download_s", C.c_double),
        ("setup_s", C.c_double), ("sweep_s", C.c_double), ("lanczos_ms", C.c_double),
        ("split_ms", C.c_double), ("env_ms", C.c_double), ("matvec_flops", C.c_double),
        ("total_gemm_flops", C.c_double), ("matvecs", C.c_long), ("kernel_launches", C.c_long),
        ("sweeps", C.c_int), ("max_bond_dim", C.c_int64), ("svd_max_sweeps", C.c_int),
        ("host_plan_s", C.c_double), ("plan_hits", C.c_long), ("plan_misses", C.c_long),
        ("svd_flops", C.c_double), ("near_ties", C.c_long),
    ]


def load(path: str = LIB_PATH) -> C.CDLL:
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing; build it with `python -m chemtensor_gb300.build`")
    lib = C.CDLL(path)
    P = C.c_void_p
    lib.dmrg_twosite.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_int64, P, P, P]
    lib.dmrg_twosite.restype = C.c_int
    lib.dmrg_singlesite.argtypes = [P, C.c_int, C.c_int, P, P]
    lib.dmrg_singlesite.restype = C.c_int
    lib.ctgpu_set_precision.argtypes = [C.c_int]
    lib.ctgpu_set_reduced_environments.argtypes = [C.c_int]
    lib.ctgpu_set_device.argtypes = [C.c_int]
    lib.ctgpu_get_last_stats.argtypes = [P]
    lib.ctgpu_last_error.restype = C.c_char_p
    lib.ctgpu_construct_random_mps.argtypes = [C.c_int, C.c_int64, P, C.c_int32, C.c_int64, C.c_uint64, P]
    lib.ctgpu_randn_sequence.argtypes = [C.c_uint64, C.c_int, P]
    lib.ctgpu_randn_sequence.restype = None
    lib.ctgpu_block_sparse_tensor_dot.argtypes = [P, C.c_int, P, C.c_int, C.c_int, P]
    lib.ctgpu_block_sparse_tensor_transpose.argtypes = [P, P, P]
    lib.ctgpu_apply_local_hamiltonian.argtypes = [P] * 5
    lib.ctgpu_time_local_hamiltonian.argtypes = [P, P, P, P, C.c_int, P, P]
    lib.ctgpu_clear_plan_cache.argtypes = []
    lib.ctgpu_contraction_operator_step_left.argtypes = [P] * 4
    lib.ctgpu_contraction_operator_step_right.argtypes = [P] * 4
    lib.ctgpu_block_sparse_tensor_svd_values.argtypes = [P, P, P]
    lib.ctgpu_block_sparse_tensor_qr.argtypes = [P, C.c_int, P, P]
    lib.ctgpu_construct_spin_molecular_mpo.argtypes = [C.c_int, P, P, P]
    lib.ctgpu_mps_vdot.argtypes = [P, P, P]
    lib.ctgpu_device_memory.argtypes = [C.c_int, P, P]
    lib.ctgpu_mps_norm.argtypes = [P, P]
    lib.ctgpu_block_sparse_tensor_rq.argtypes = [P, C.c_int, P, P]
    lib.ctgpu_delete_block_sparse_tensor.argtypes = [P]
    lib.ctgpu_delete_block_sparse_tensor.restype = None
    lib.ctgpu_set_profiling.argtypes = [C.c_int, C.c_int]
    lib.ctgpu_set_l2_flush_bytes.argtypes = [C.c_int64]
    lib.ctgpu_set_l2_flush_bytes.restype = None
    lib.ctgpu_get_sweep_times.argtypes = [P, P, C.c_int]
    lib.ctgpu_get_kernel_profile.argtypes = [C.c_int, P, P, P, P]
    lib.ctgpu_measure_fp64_tflops.restype = C.c_double
    lib.ctgpu_get_bond_singular_values.argtypes = [C.c_int, P, C.c_int64]
    lib.ctgpu_get_bond_singular_values.restype = C.c_int64
    lib.ctgpu_tile_tuning_report.argtypes = [C.c_char_p, C.c_int]
    lib.ctgpu_set_tc_tile_width.argtypes = [C.c_int]
    lib.ctgpu_set_tc_wait_limit.argtypes = [C.c_longlong]
    lib.ctgpu_set_tc_wait_limit.restype = None
    lib.ctgpu_inject_failure.argtypes = [C.c_int, C.c_int]
    lib.ctgpu_tridiag_lowest.argtypes = [P, P, C.c_int, P, P]
    lib.ctgpu_mpo_inner_product.argtypes = [P, P, P, P]
    lib.ctgpu_set_final_fp64_sweeps.argtypes = [C.c_int]
    return lib


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = load()
    return _lib


def last_error() -> str:
    return lib().ctgpu_last_error().decode()


def last_stats() -> dict:
    s = Stats()
    lib().ctgpu_get_last_stats(C.byref(s))
    return {k: getattr(s, k) for k, _ in Stats._fields_}


def sweep_times():
    n = lib().ctgpu_get_sweep_times(None, None, 0)
    ms = np.zeros(max(n, 1))
    la = np.zeros(max(n, 1), dtype=np.int64)
    lib().ctgpu_get_sweep_times(ms.ctypes.data, la.ctypes.data, n)
    return ms[:n], la[:n]


def kernel_profile() -> dict:
    out = {}
    for i, name in enumerate(KERNEL_CLASSES):
        la, ms, fl, by = C.c_long(), C.c_double(), C.c_double(), C.c_double()
        lib().ctgpu_get_kernel_profile(i, C.byref(la), C.byref(ms), C.byref(fl), C.byref(by))
        out[name] = {"launches": la.value, "ms": ms.value, "flops": fl.value, "bytes": by.value}
    return out


def bond_singular_values(bond: int) -> np.ndarray | None:
    """Retained singular values of the last split at `bond` in this thread's last dmrg_twosite call."""
    n = lib().ctgpu_get_bond_singular_values(bond, None, 0)
    if n < 0:
        return None
    out = np.zeros(max(n, 1))
    lib().ctgpu_get_bond_singular_values(bond, out.ctypes.data, n)
    return out[:n]


def tile_tuning() -> list:
    """The GEMM autotuner's choices so far: [{key, bn (0 = FP64), ms: [64, 128, 256, fp64], source}]."""
    n = lib().ctgpu_tile_tuning_report(None, 0)
    buf = C.create_string_buffer(max(n, 0) + 1)
    lib().ctgpu_tile_tuning_report(buf, len(buf))
    out = []
    for line in buf.value.decode().splitlines():
        p = line.split()
        if len(p) == 7:
            out.append({"key": p[0], "bn": int(p[1]), "ms": [float(x) for x in p[2:6]], "source": p[6]})
    return out


def set_precision(p: int) -> int:
    """Select the block-GEMM arithmetic for later calls; returns the previous setting."""
    old = lib().ctgpu_set_precision(int(p))
    if old < 0:
        raise ValueError(f"unknown precision {p}")
    return old


def random_mps(nsites: int, d: int, qsite, qnum_sector: int, max_vdim: int, seed: int) -> cs.MPS:
    """Reference-identical seeded random MPS as a C struct (caller frees with free_mps)."""
    q = np.ascontiguousarray(qsite, dtype=np.int32)
    m = cs.MPS()
    ret = lib().ctgpu_construct_random_mps(nsites, d, q.ctypes.data, int(qnum_sector), max_vdim, seed, C.byref(m))
    if ret != 0:
        raise ValueError("invalid random MPS parameters")
    return m


def dmrg_twosite(mpo: cs.MPO, psi: cs.MPS, num_sweeps: int, maxiter_lanczos: int, tol_split: float, max_vdim: int):
    """Call the C-ABI dmrg_twosite; psi is updated in place. Returns (ret, en_sweeps, entropy)."""
    en = np.zeros(max(num_sweeps, 1))
    ent = np.zeros(max(mpo.nsites - 1, 1))
    ret = lib().dmrg_twosite(C.byref(mpo), num_sweeps, maxiter_lanczos, tol_split, max_vdim, C.byref(psi),
                             en.ctypes.data, ent.ctypes.data)
    return ret, en[:num_sweeps], ent[:mpo.nsites - 1]


def dmrg_singlesite(mpo: cs.MPO, psi: cs.MPS, num_sweeps: int, maxiter_lanczos: int):
    """Call the C-ABI dmrg_singlesite; psi is updated in place. Returns (ret, en_sweeps)."""
    en = np.zeros(max(num_sweeps, 1))
    ret = lib().dmrg_singlesite(C.byref(mpo), num_sweeps, maxiter_lanczos, C.byref(psi), en.ctypes.data)
    return ret, en[:num_sweeps]
