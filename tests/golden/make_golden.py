"""Generate the golden fixtures in this directory from the chemtensor reference.

The reference is compiled from its own sources by ``make -C oracle ref`` into
oracle/_ref/libct_ref.so (only where the reference checkout exists); this script
drives it through ctypes and stores, as .npz:

* the reference's own inputs: MPOs built by its Hamiltonian assembly code and
  seeded random MPS from construct_random_mps (src/state/mps.c:93);
* the reference's outputs of dmrg_twosite (src/algorithm/dmrg.c:262): energies
  per sweep, entanglement entropies and the optimised MPS; and of dmrg_singlesite
  (src/algorithm/dmrg.c:155): energies per sweep and the optimised MPS;
* pseudo-random sequences of its PCG32x2 + Box-Muller generator (src/util/rng.c);
* single-operation pins: apply_local_hamiltonian and the environment updates on
  one bond (src/algorithm/chain_ops.c); block_sparse_tensor_qr / _rq on random
  block-sparse matrices (src/tensor/block_sparse_tensor.c).

* the spin-orbital molecular Hamiltonian MPO (src/operator/hamiltonian.c:2768) and a
  dmrg_twosite run on it.

* complex128 runs of dmrg_twosite and dmrg_singlesite (complex gauge on the MPO bonds,
  complex random start states).

Run from the repository root:  python tests/golden/make_golden.py [singlesite|qr|molecular|complex]
(with an argument, only that group of fixtures is written).
"""

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from chemtensor_gb300 import ctstructs as cs  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libct_ref.so"))
ref.dmrg_twosite.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
ref.dmrg_singlesite.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
ref.ref_heisenberg_mpo.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_void_p]
ref.ref_hubbard_mpo.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_void_p]
ref.ref_random_mps.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p]
ref.ref_randn_sequence.argtypes = [C.c_uint64, C.c_int, C.c_void_p]
ref.ref_local_hamiltonian_setup.argtypes = [C.c_void_p] * 2 + [C.c_int] + [C.c_void_p] * 4
ref.apply_local_hamiltonian.argtypes = [C.c_void_p] * 5
ref.contraction_operator_step_left.argtypes = [C.c_void_p] * 5
ref.contraction_operator_step_right.argtypes = [C.c_void_p] * 5
ref.ref_spin_molecular_mpo.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
ref.block_sparse_tensor_qr.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
ref.block_sparse_tensor_rq.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]

HUB_QSITE = [(n << 16) + s for n, s in [(0, 0), (1, -1), (1, 1), (2, 0)]]


def mpo(model, L, **kw):
    m = cs.MPO()
    if model == "heisenberg":
        ref.ref_heisenberg_mpo(L, kw.get("J", 1.0), kw.get("Delta", 1.0), kw.get("h", 0.0), C.byref(m))
    else:
        ref.ref_hubbard_mpo(L, kw.get("t", 1.0), kw.get("u", 4.0), kw.get("mu", 0.0), C.byref(m))
    return m


def random_mps(L, qsite, sector, D, seed):
    p = cs.MPS()
    qa = (C.c_int32 * len(qsite))(*qsite)
    ref.ref_random_mps(1, L, len(qsite), qa, sector, D, seed, C.byref(p))
    return p


def dmrg_case(name, model, L, D, sweeps, maxiter, tol, seed, **kw):
    H = mpo(model, L, **kw)
    if model == "heisenberg":
        qsite, sector = [1, -1], 0
    else:
        qsite, sector = HUB_QSITE, (L << 16)
    psi = random_mps(L, qsite, sector, D, seed)
    arrays = {}
    arrays.update(cs.chain_to_arrays("H", cs.read_mpo(H)))
    arrays.update(cs.chain_to_arrays("psi0", cs.read_mps(psi)))
    en = (C.c_double * sweeps)()
    ent = (C.c_double * (L - 1))()
    ret = ref.dmrg_twosite(C.byref(H), sweeps, maxiter, tol, D, C.byref(psi), en, ent)
    assert ret == 0
    arrays.update(cs.chain_to_arrays("psi", cs.read_mps(psi)))
    arrays.update(en_sweeps=np.array(en), entropy=np.array(ent),
                  params=np.array([L, D, sweeps, maxiter], dtype=np.int64), tol_split=np.array(tol),
                  seed=np.array(seed), model=np.array(model))
    np.savez_compressed(os.path.join(OUT, name), **arrays)
    print(name, "E =", en[sweeps - 1])
    return H, psi


def dmrg1_case(name, model, L, D, sweeps, maxiter, seed, **kw):
    H = mpo(model, L, **kw)
    if model == "heisenberg":
        qsite, sector = [1, -1], 0
    else:
        qsite, sector = HUB_QSITE, (L << 16)
    psi = random_mps(L, qsite, sector, D, seed)
    arrays = {}
    arrays.update(cs.chain_to_arrays("H", cs.read_mpo(H)))
    arrays.update(cs.chain_to_arrays("psi0", cs.read_mps(psi)))
    en = (C.c_double * sweeps)()
    ret = ref.dmrg_singlesite(C.byref(H), sweeps, maxiter, C.byref(psi), en)
    assert ret == 0
    arrays.update(cs.chain_to_arrays("psi", cs.read_mps(psi)))
    arrays.update(en_sweeps=np.array(en), params=np.array([L, D, sweeps, maxiter], dtype=np.int64),
                  seed=np.array(seed), model=np.array(model))
    np.savez_compressed(os.path.join(OUT, name), **arrays)
    print(name, "E =", en[sweeps - 1])


def singlesite_cases():
    # dmrg_singlesite end to end (bond dimensions fixed by the start state)
    dmrg1_case("dmrg1_heisenberg_L12_D16.npz", "heisenberg", 12, 16, 4, 5, 3, Delta=0.7)
    dmrg1_case("dmrg1_hubbard_L8_D24.npz", "hubbard", 8, 24, 3, 5, 11, u=3.0)


def qr_cases():
    """block_sparse_tensor_qr / _rq (src/tensor/block_sparse_tensor.c:2402-2676), QR_REDUCED, on
    random block-sparse matrices: tall and wide blocks, a zero column, and a matrix without blocks."""
    rng = np.random.default_rng(2024)
    arrays = {}
    specs = {
        "m0": ((40, 30), (1, -1), 3),
        "m1": ((30, 52), (-1, 1), 2),
        "m2": ((64, 64), (1, 1), 1),
        "m3": ((17, 9), (1, -1), 4),
    }
    for tag, (dims, dirs, qr_) in specs.items():
        qn = [rng.integers(-qr_, qr_ + 1, size=d).astype(np.int32) for d in dims]
        t = cs.BlockSparse(dims, dirs, qn)
        for i, idx in enumerate(t.allowed):
            b = rng.standard_normal(t.block_shape(idx))
            if i == 0 and b.shape[1] > 2:
                b[:, 1] = 0.0
            t.blocks[idx] = b
        arrays.update(cs.bst_to_arrays(tag, t))
    # no allowed blocks: dummy factors
    t = cs.BlockSparse((5, 6), (1, -1), [np.zeros(5, np.int32), np.ones(6, np.int32)])
    assert not t.allowed
    arrays.update(cs.bst_to_arrays("m4", t))
    for tag in ["m0", "m1", "m2", "m3", "m4"]:
        a = cs.BlockSparseTensor()
        cs.write_bst(cs.bst_from_arrays(tag, arrays), a)
        q, r = cs.BlockSparseTensor(), cs.BlockSparseTensor()
        assert ref.block_sparse_tensor_qr(C.byref(a), 0, C.byref(q), C.byref(r)) == 0
        arrays.update(cs.bst_to_arrays(tag + "_qr_q", cs.read_bst(q)))
        arrays.update(cs.bst_to_arrays(tag + "_qr_r", cs.read_bst(r)))
        r2, q2 = cs.BlockSparseTensor(), cs.BlockSparseTensor()
        assert ref.block_sparse_tensor_rq(C.byref(a), 0, C.byref(r2), C.byref(q2)) == 0
        arrays.update(cs.bst_to_arrays(tag + "_rq_r", cs.read_bst(r2)))
        arrays.update(cs.bst_to_arrays(tag + "_rq_q", cs.read_bst(q2)))
        for x in (a, q, r, r2, q2):
            cs.free_bst(x)
    np.savez_compressed(os.path.join(OUT, "qr_rq_blocks.npz"), **arrays)
    print("qr_rq_blocks.npz", len(arrays), "arrays")


def molecular_cases():
    """construct_spin_molecular_hamiltonian_mpo_assembly(optimize=false) + mpo_from_assembly
    (src/operator/hamiltonian.c:2768-2979): the full MPO for n = 4 with general (non-symmetric)
    coefficients, and for n = 24 with the synthetic integrals of the molecular workload the bond
    quantum numbers and stored entries per site; plus a small dmrg_twosite run on n = 6."""
    sys.path.insert(0, ROOT)
    from chemtensor_gb300 import workloads as wl

    def build(tk, vi):
        m = cs.MPO()
        n = tk.shape[0]
        ref.ref_spin_molecular_mpo(n, np.ascontiguousarray(tk).ctypes.data, np.ascontiguousarray(vi).ctypes.data, 0,
                                   C.byref(m))
        return m

    arrays = {}
    rng = np.random.default_rng(205)
    tk, vi = rng.standard_normal((4, 4)), rng.standard_normal((4, 4, 4, 4))
    arrays.update(tkin4=tk, vint4=vi)
    arrays.update(cs.chain_to_arrays("H4", cs.read_mpo(build(tk, vi))))
    # odd and small orbital counts (pair states change sides at an odd bond)
    for n in (1, 2, 5):
        tk, vi = rng.standard_normal((n, n)), rng.standard_normal((n, n, n, n))
        arrays.update({f"tkin{n}": tk, f"vint{n}": vi})
        arrays.update(cs.chain_to_arrays(f"H{n}", cs.read_mpo(build(tk, vi))))
    tk, vi = wl.molecular_integrals(24, 7)
    ch = cs.read_mpo(build(tk, vi))
    for i, t in enumerate(ch.tensors):
        arrays[f"q24_bond{i}"] = np.sort(np.asarray(t.qnums_logical[0], dtype=np.int32))
        arrays[f"nnz24_site{i}"] = np.array(t.num_elements_blocks())
    np.savez_compressed(os.path.join(OUT, "spin_molecular_mpo.npz"), **arrays)
    print("spin_molecular_mpo.npz")

    # dmrg_twosite on a 6-orbital molecular Hamiltonian (the workload's integrals at n = 6)
    L, D, sweeps, maxiter, tol, seed = 6, 32, 3, 5, 1e-10, 17
    tk, vi = wl.molecular_integrals(L, 3)
    H = build(tk, vi)
    psi = random_mps(L, HUB_QSITE, (L << 16), D, seed)
    arrays = {"tkin": tk, "vint": vi}
    arrays.update(cs.chain_to_arrays("H", cs.read_mpo(H)))
    arrays.update(cs.chain_to_arrays("psi0", cs.read_mps(psi)))
    en = (C.c_double * sweeps)()
    ent = (C.c_double * (L - 1))()
    assert ref.dmrg_twosite(C.byref(H), sweeps, maxiter, tol, D, C.byref(psi), en, ent) == 0
    arrays.update(cs.chain_to_arrays("psi", cs.read_mps(psi)))
    arrays.update(en_sweeps=np.array(en), entropy=np.array(ent),
                  params=np.array([L, D, sweeps, maxiter], dtype=np.int64), tol_split=np.array(tol),
                  seed=np.array(seed), model=np.array("molecular"))
    np.savez_compressed(os.path.join(OUT, "dmrg_molecular_n6_D32.npz"), **arrays)
    print("dmrg_molecular_n6_D32.npz E =", en[sweeps - 1])


def complex_mpo(model, L, seed, **kw):
    """The reference's real MPO turned complex by random phases on its virtual bonds
    (W_i[..., k] *= e^{i t_k}, W_{i+1}[k, ...] *= e^{-i t_k}): the same Hermitian operator,
    complex128 entries throughout."""
    ch = cs.read_mpo(mpo(model, L, **kw))
    rng = np.random.default_rng(seed)
    ts = []
    for t in ch.tensors:
        z = cs.BlockSparse(t.dim_logical, t.axis_dir, t.qnums_logical, dtype=cs.CT_DOUBLE_COMPLEX)
        for idx, b in t.blocks.items():
            z.blocks[idx] = b.astype(np.complex128)
        ts.append(z)
    for i in range(L - 1):
        ph = np.exp(1j * rng.uniform(0.0, 2 * np.pi, size=ts[i].dim_logical[3]))
        for t, ax, sgn in ((ts[i], 3, 1), (ts[i + 1], 0, -1)):
            for idx in list(t.blocks):
                sel = np.nonzero(t.qnums_logical[ax] == t.qnums_blocks[ax][idx[ax]])[0]
                shape = [1, 1, 1, 1]
                shape[ax] = len(sel)
                t.blocks[idx] = t.blocks[idx] * (ph[sel] if sgn > 0 else np.conj(ph[sel])).reshape(shape)
    return cs.Chain(ts, ch.qsite, ch.d)


def complex_cases():
    """dmrg_twosite and dmrg_singlesite in complex128 (CT_DOUBLE_COMPLEX): Fermi-Hubbard chain with
    a complex gauge on the MPO bonds and complex random start states (construct_random_mps)."""
    for name, L, D, sweeps, maxiter, seed, single in (("dmrg_complex_hubbard_L6_D32.npz", 6, 32, 3, 5, 29, False),
                                                      ("dmrg1_complex_hubbard_L6_D24.npz", 6, 24, 3, 5, 31, True)):
        Hc = complex_mpo("hubbard", L, seed + 100, u=3.0)
        p = cs.MPS()
        qa = (C.c_int32 * 4)(*HUB_QSITE)
        ref.ref_random_mps(cs.CT_DOUBLE_COMPLEX, L, 4, qa, (L << 16), D, seed, C.byref(p))
        arrays = {}
        arrays.update(cs.chain_to_arrays("H", Hc))
        arrays.update(cs.chain_to_arrays("psi0", cs.read_mps(p)))
        cH = cs.make_c_mpo(Hc)
        en = (C.c_double * sweeps)()
        ent = (C.c_double * (L - 1))()
        if single:
            assert ref.dmrg_singlesite(C.byref(cH), sweeps, maxiter, C.byref(p), en) == 0
        else:
            assert ref.dmrg_twosite(C.byref(cH), sweeps, maxiter, 1e-10, D, C.byref(p), en, ent) == 0
            arrays.update(entropy=np.array(ent))
        arrays.update(cs.chain_to_arrays("psi", cs.read_mps(p)))
        arrays.update(en_sweeps=np.array(en), params=np.array([L, D, sweeps, maxiter], dtype=np.int64),
                      tol_split=np.array(1e-10), seed=np.array(seed), model=np.array("hubbard complex gauge"))
        np.savez_compressed(os.path.join(OUT, name), **arrays)
        print(name, "E =", en[sweeps - 1])


def local_ops_case(name, model, L, D, seed, ibond, **kw):
    """Reference inputs/outputs of one local-H apply and one left / right environment step."""
    H = mpo(model, L, **kw)
    qsite, sector = ([1, -1], 0) if model == "heisenberg" else (HUB_QSITE, L << 16)
    psi = random_mps(L, qsite, sector, D, seed)
    h2, le, re, a2, b = (cs.BlockSparseTensor() for _ in range(5))
    ref.ref_local_hamiltonian_setup(C.byref(H), C.byref(psi), ibond, C.byref(h2), C.byref(le), C.byref(re), C.byref(a2))
    ref.apply_local_hamiltonian(C.byref(a2), C.byref(h2), C.byref(le), C.byref(re), C.byref(b))
    lnext, rnext = cs.BlockSparseTensor(), cs.BlockSparseTensor()
    A = psi.a[ibond]
    ref.contraction_operator_step_left(C.byref(A), C.byref(A), C.byref(H.a[ibond]), C.byref(le), C.byref(lnext))
    B = psi.a[ibond + 1]
    ref.contraction_operator_step_right(C.byref(B), C.byref(B), C.byref(H.a[ibond + 1]), C.byref(re), C.byref(rnext))
    arrays = {}
    for p, t in [("h2", h2), ("l", le), ("r", re), ("a", a2), ("b", b), ("lnext", lnext), ("rnext", rnext)]:
        arrays.update(cs.bst_to_arrays(p, cs.read_bst(t)))
    arrays.update(cs.bst_to_arrays("A", cs.read_bst(A)))
    arrays.update(cs.bst_to_arrays("B", cs.read_bst(B)))
    arrays.update(cs.bst_to_arrays("W", cs.read_bst(H.a[ibond])))
    arrays.update(cs.bst_to_arrays("W1", cs.read_bst(H.a[ibond + 1])))
    np.savez_compressed(os.path.join(OUT, name), **arrays)
    print(name, "entries a/b:", cs.read_bst(a2).num_elements_blocks())


def main():
    # PCG32x2 + Box-Muller sequences (src/util/rng.c:15-125)
    seqs = {}
    for seed in (0, 42, 7, 12345678901):
        buf = (C.c_double * 2000)()
        ref.ref_randn_sequence(seed, 2000, buf)
        seqs[f"randn_{seed}"] = np.array(buf)
    np.savez_compressed(os.path.join(OUT, "rng_sequences.npz"), **seqs)

    # construct_random_mps outputs (src/state/mps.c:93-175), including Floyd sampling of bond quantum numbers
    arrays = {}
    for tag, (L, qs, sec, D, seed) in {
        "heis_L12_D8_s1": (12, [1, -1], 0, 8, 1),
        "hub_L8_D24_s3": (8, HUB_QSITE, 8 << 16, 24, 3),
        "hub_L10_D16_s42": (10, HUB_QSITE, (10 << 16) + 2, 16, 42),
    }.items():
        p = random_mps(L, qs, sec, D, seed)
        arrays.update(cs.chain_to_arrays(tag, cs.read_mps(p)))
        arrays[f"{tag}_params"] = np.array([L, sec, D, seed], dtype=np.int64)
        arrays[f"{tag}_qsite"] = np.array(qs, dtype=np.int32)
    np.savez_compressed(os.path.join(OUT, "random_mps.npz"), **arrays)

    # MPOs built by the reference's assembly code (for operator equality of the builders)
    arrays = {}
    arrays.update(cs.chain_to_arrays("heis6", cs.read_mpo(mpo("heisenberg", 6, J=1.0, Delta=0.8, h=0.3))))
    arrays.update(cs.chain_to_arrays("hub4", cs.read_mpo(mpo("hubbard", 4, t=1.0, u=4.0, mu=0.3))))
    np.savez_compressed(os.path.join(OUT, "mpo_reference.npz"), **arrays)

    # dmrg_twosite end to end
    dmrg_case("dmrg_heisenberg_L20_D32.npz", "heisenberg", 20, 32, 6, 5, 1e-10, 42)
    dmrg_case("dmrg_heisenberg_L10_D16.npz", "heisenberg", 10, 16, 3, 5, 1e-10, 7, Delta=0.5, h=0.1)
    dmrg_case("dmrg_hubbard_L8_D32.npz", "hubbard", 8, 32, 4, 5, 1e-10, 42)
    dmrg_case("dmrg_hubbard_L12_D48.npz", "hubbard", 12, 48, 2, 7, 1e-10, 5, u=2.0, mu=0.25)

    # single operations on one bond
    local_ops_case("local_ops_heisenberg_L12.npz", "heisenberg", 12, 16, 11, 5)
    local_ops_case("local_ops_hubbard_L8.npz", "hubbard", 8, 32, 13, 3)


if __name__ == "__main__":
    if sys.argv[1:] == ["singlesite"]:
        singlesite_cases()
    elif sys.argv[1:] == ["qr"]:
        qr_cases()
    elif sys.argv[1:] == ["molecular"]:
        molecular_cases()
    elif sys.argv[1:] == ["complex"]:
        complex_cases()
    else:
        main()
        singlesite_cases()
        qr_cases()
        molecular_cases()
        complex_cases()
