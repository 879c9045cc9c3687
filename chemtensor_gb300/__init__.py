"""GB300-native implementation of chemtensor's two-site DMRG path.

The compute path is libctgpu.so (CUDA kernels for sm_103a behind the C ABI in
include/ctgpu.h, whose dmrg_twosite is a drop-in for the reference's). This
package holds the host-side mirror of the reference's Python entry point and
the input builders; it has no compute fallback.
"""

from . import ctstructs, hamiltonians  # noqa: F401

__all__ = ["ctstructs", "hamiltonians", "dmrg"]


def dmrg(mpo, num_sweeps=5, maxiter_lanczos=20, tol_split=1e-10, max_vdim=256, qnum_sector=0, rng_seed=42):
    """Mirror of the reference's Python ``chemtensor.dmrg`` (python/pymodule.c:3238-3359):
    build a seeded random MPS in the requested sector, run two-site DMRG on the GPU and
    return (MPS as a ctstructs.Chain, list of sweep energies, list of bond entropies).

    ``mpo`` is a ctstructs.Chain (for example from chemtensor_gb300.hamiltonians).
    Raises ValueError on invalid arguments and RuntimeError if the solver fails, as the
    reference binding does.
    """
    from . import native

    if num_sweeps <= 0:
        raise ValueError("'num_sweeps' must be a positive integer")
    if maxiter_lanczos <= 0:
        raise ValueError("'maxiter_lanczos' must be a positive integer")
    if tol_split < 0 or tol_split > 1:
        raise ValueError("'tol_split' must be a number between 0 and 1")
    if max_vdim <= 0:
        raise ValueError("'max_vdim' must be a positive integer")
    c_mpo = ctstructs.make_c_mpo(mpo)
    c_mps = native.random_mps(mpo.nsites, mpo.d, mpo.qsite, qnum_sector, max_vdim, rng_seed)
    try:
        ret, en, ent = native.dmrg_twosite(c_mpo, c_mps, num_sweeps, maxiter_lanczos, tol_split, max_vdim)
        if ret < 0:
            raise RuntimeError(f"'dmrg_twosite' failed internally: {native.last_error() or ret}")
        return ctstructs.read_mps(c_mps), list(en), list(ent)
    finally:
        ctstructs.free_mps(c_mps)
        ctstructs.free_mpo(c_mpo)
