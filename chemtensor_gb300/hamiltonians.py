"""MPO builders for the lattice Hamiltonians of the DMRG workloads (host-side inputs).

Each builder writes the Hamiltonian as a finite-state-machine MPO with bond
states "nothing placed yet", one state per open two-site operator, and
"everything placed". The operator is the same as the reference's
(src/operator/hamiltonian.c), which reaches it through its MPO-graph
assembly; only the gauge of the virtual MPO bonds differs, which leaves the
local effective Hamiltonians of DMRG unchanged.

Site tensors have legs (Dw_left, d, d, Dw_right), directions
(OUT, OUT, IN, IN) and W[wl, s, s', wr] = <s| op |s'> (mpo.c:48, :96-117).
"""

from __future__ import annotations

import numpy as np

from . import ctstructs as cs


def encode_quantum_number_pair(qa: int, qb: int) -> int:
    """(N, 2 Sz) -> single quantum number (include/tensor/qnumber.h:47-52)."""
    return (int(qa) << 16) + int(qb)


def dense_to_block_sparse(dense: np.ndarray, axis_dir, qnums) -> cs.BlockSparse:
    """Cut a dense array into the blocks allowed by the quantum numbers; entries
    outside the allowed blocks must vanish."""
    t = cs.BlockSparse(dense.shape, axis_dir, qnums)
    maps = [[np.nonzero(t.qnums_logical[i] == q)[0] for q in t.qnums_blocks[i]] for i in range(t.ndim)]
    covered = np.zeros(dense.shape, dtype=bool)
    for idx in t.allowed:
        sel = np.ix_(*[maps[i][j] for i, j in enumerate(idx)])
        t.blocks[idx] = np.ascontiguousarray(dense[sel], dtype=np.float64)
        covered[sel] = True
    if np.any(dense[~covered] != 0):
        raise ValueError("dense tensor has entries that violate quantum number conservation")
    return t


def _fsm_mpo(nsites: int, d: int, qsite, bond_q, wmid) -> cs.Chain:
    """Assemble site tensors from the bulk FSM tensor 'wmid' (Dw, d, d, Dw): the first
    site keeps the start row, the last site the final column."""
    dw = len(bond_q)
    dirs = (cs.TENSOR_AXIS_OUT, cs.TENSOR_AXIS_OUT, cs.TENSOR_AXIS_IN, cs.TENSOR_AXIS_IN)
    tensors = []
    for i in range(nsites):
        w = wmid
        ql, qr = list(bond_q), list(bond_q)
        if i == 0:
            w = w[:1]
            ql = [bond_q[0]]
        if i == nsites - 1:
            w = w[..., dw - 1:]
            qr = [bond_q[dw - 1]]
        tensors.append(dense_to_block_sparse(np.ascontiguousarray(w), dirs, [ql, qsite, qsite, qr]))
    return cs.Chain(tensors, np.asarray(qsite, dtype=np.int32), d)


def heisenberg_xxz_1d(nsites: int, J: float, D: float, h: float) -> cs.Chain:
    """sum_i J (X_i X_{i+1} + Y_i Y_{i+1} + D Z_i Z_{i+1}) - h sum_i Z_i with spin-1/2
    operators, i.e. J/2 (S+S- + S-S+) + J D Sz Sz - h Sz
    (construct_heisenberg_xxz_1d_mpo_assembly, src/operator/hamiltonian.c:102-155).
    Local basis (up, down) with quantum numbers 2 Sz = (1, -1)."""
    assert nsites >= 2
    qsite = [1, -1]
    I2 = np.eye(2)
    sup = np.array([[0.0, 1.0], [0.0, 0.0]])
    sdn = np.array([[0.0, 0.0], [1.0, 0.0]])
    sz = np.array([[0.5, 0.0], [0.0, -0.5]])
    # bond states: start, S+ open, S- open, Sz open, done
    bond_q = [0, 2, -2, 0, 0]
    w = np.zeros((5, 2, 2, 5))
    w[0, :, :, 0] = I2
    w[0, :, :, 1] = sup
    w[0, :, :, 2] = sdn
    w[0, :, :, 3] = sz
    w[0, :, :, 4] = -h * sz
    w[1, :, :, 4] = 0.5 * J * sdn
    w[2, :, :, 4] = 0.5 * J * sup
    w[3, :, :, 4] = J * D * sz
    w[4, :, :, 4] = I2
    return _fsm_mpo(nsites, 2, qsite, bond_q, w)


HUBBARD_QSITE = [encode_quantum_number_pair(n, s) for n, s in [(0, 0), (1, -1), (1, 1), (2, 0)]]


def fermi_hubbard_1d(nsites: int, t: float, u: float, mu: float) -> cs.Chain:
    """-t sum_{i,sigma} (c^dag_{i sigma} c_{i+1 sigma} + h.c.) + u sum_i (n_up - 1/2)(n_dn - 1/2)
    - mu sum_i (n_up + n_dn), Jordan-Wigner ordered (up_i, dn_i, up_{i+1}, ...)
    (construct_fermi_hubbard_1d_mpo_assembly, src/operator/hamiltonian.c:240-375).
    Local basis |0>, |dn>, |up>, |up dn> with quantum numbers encode(N, 2 Sz)."""
    assert nsites >= 2
    I2 = np.eye(2)
    cdag = np.array([[0.0, 0.0], [1.0, 0.0]])
    cann = np.array([[0.0, 1.0], [0.0, 0.0]])
    Z = np.diag([1.0, -1.0])
    kron = np.kron
    CI, AI, CZ, AZ = kron(cdag, I2), kron(cann, I2), kron(cdag, Z), kron(cann, Z)
    IC, IA, ZC, ZA = kron(I2, cdag), kron(I2, cann), kron(Z, cdag), kron(Z, cann)
    Nt = np.diag([0.0, 1.0, 1.0, 2.0])
    NI = np.diag([0.25, -0.25, -0.25, 0.25])
    e = encode_quantum_number_pair
    # bond states: start, (up created | Z), (up annihilated | Z), (dn created), (dn annihilated), done
    bond_q = [0, e(1, 1), e(-1, -1), e(1, -1), e(-1, 1), 0]
    w = np.zeros((6, 4, 4, 6))
    w[0, :, :, 0] = np.eye(4)
    w[0, :, :, 1] = CZ
    w[1, :, :, 5] = -t * AI
    w[0, :, :, 2] = AZ
    w[2, :, :, 5] = -t * CI
    w[0, :, :, 3] = IC
    w[3, :, :, 5] = -t * ZA
    w[0, :, :, 4] = IA
    w[4, :, :, 5] = -t * ZC
    w[0, :, :, 5] = -mu * Nt + u * NI
    w[5, :, :, 5] = np.eye(4)
    return _fsm_mpo(nsites, 4, HUBBARD_QSITE, bond_q, w)


def mpo_to_matrix(ch: cs.Chain) -> np.ndarray:
    """Dense operator of a (small) MPO: contract the virtual bonds, physical row index
    = output states, column index = input states (for tests)."""
    acc = ch.tensors[0].to_dense()          # (1, d, d, D)
    acc = acc[0]                            # (d, d, D)
    for t in ch.tensors[1:]:
        w = t.to_dense()                    # (D, d, d, D')
        acc = np.einsum("abx,xcdy->acbdy", acc, w)
        s = acc.shape
        acc = acc.reshape(s[0] * s[1], s[2] * s[3], s[4])
    return acc[..., 0]


def spin_molecular(tkin: np.ndarray, vint: np.ndarray) -> cs.Chain:
    """Spin-orbital molecular Hamiltonian (physicists' order of vint) as an MPO, built by the
    C-ABI ctgpu_construct_spin_molecular_mpo (host code of libctgpu.so); same operator, bond
    dimensions and bond quantum numbers as the reference's
    construct_spin_molecular_hamiltonian_mpo_assembly(tkin, vint, optimize=false)
    (src/operator/hamiltonian.c:2768-2979)."""
    import ctypes as C

    from . import native
    tkin = np.ascontiguousarray(tkin, dtype=np.float64)
    vint = np.ascontiguousarray(vint, dtype=np.float64)
    n = tkin.shape[0]
    if tkin.shape != (n, n) or vint.shape != (n, n, n, n):
        raise ValueError("tkin must be n x n and vint n x n x n x n")
    m = cs.MPO()
    if native.lib().ctgpu_construct_spin_molecular_mpo(n, tkin.ctypes.data, vint.ctypes.data, C.byref(m)) != 0:
        raise RuntimeError(native.last_error())
    ch = cs.read_mpo(m)
    cs.free_mpo(m)
    return ch
