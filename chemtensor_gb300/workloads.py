"""Synthetic inputs of the local-Hamiltonian microbenchmark.

Two-site wavefunction a (D x d^2 x D), merged MPO pair h2 (Dw x d^2 x d^2 x Dw), left and right
environments l (1 x D x Dw x D) and r (D x Dw x D x 1), with the axis directions of
apply_local_hamiltonian's operands (src/algorithm/chain_ops.c:353-390). The bond of dimension D
is split over nsec quantum-number sectors q = -(nsec-1)/2 .. (nsec-1)/2 whose sizes follow a
discretised Gaussian (width sigma sectors) centred on q = 0, rounded by largest remainders to sum
to D (sectors that round to zero are absent); d = 4 site states with charges (-1, 0, 0, +1); the
MPO bond of dimension Dw carries charges 0 (Dw - 2 Dw/3 of them), +1 and -1 (Dw/3 each).
Allowed blocks hold seeded N(0, 1) entries.
"""

from __future__ import annotations

import numpy as np

from . import ctstructs as cs


def gaussian_sector_sizes(total: int, nsec: int, sigma: float) -> np.ndarray:
    """Largest-remainder rounding of total * w / sum(w), w = exp(-k^2 / (2 sigma^2))."""
    k = np.arange(nsec) - (nsec - 1) / 2
    w = np.exp(-0.5 * (k / sigma) ** 2)
    exact = total * w / w.sum()
    sizes = np.floor(exact).astype(np.int64)
    rest = total - int(sizes.sum())
    order = np.argsort(-(exact - sizes), kind="stable")
    sizes[order[:rest]] += 1
    return sizes


def _fill(t: cs.BlockSparse, rng) -> cs.BlockSparse:
    for idx in t.allowed:
        t.blocks[idx] = rng.standard_normal(t.block_shape(idx))
    return t


def local_h_microbench(D: int = 1024, nsec: int = 41, sigma: float = 6.0, Dw: int = 26, seed: int = 1):
    rng = np.random.default_rng(seed)
    sizes = gaussian_sector_sizes(D, nsec, sigma)
    q = np.arange(nsec, dtype=np.int32) - (nsec - 1) // 2
    ql = np.repeat(q, sizes)                                         # bond charges (both bonds)
    qr = ql
    qsite = np.array([-1, 0, 0, 1], dtype=np.int32)
    qpair = (qsite[:, None] + qsite[None, :]).ravel().astype(np.int32)
    nm = Dw // 3
    qw = np.concatenate([np.full(Dw - 2 * nm, 0), np.full(nm, 1), np.full(nm, -1)]).astype(np.int32)
    zero = np.zeros(1, dtype=np.int32)
    a = _fill(cs.BlockSparse((D, 16, D), (1, 1, -1), [ql, qpair, qr]), rng)
    h2 = _fill(cs.BlockSparse((Dw, 16, 16, Dw), (1, 1, -1, -1), [qw, qpair, qpair, qw]), rng)
    l = _fill(cs.BlockSparse((1, D, Dw, D), (1, -1, -1, 1), [zero, ql, qw, ql]), rng)
    r = _fill(cs.BlockSparse((D, Dw, D, 1), (1, 1, -1, -1), [qr, qw, qr, zero]), rng)
    return a, h2, l, r


def molecular_integrals(n: int = 24, seed: int = 7):
    """Synthetic molecular integrals of the molecular DMRG workload: tkin symmetric with entries
    N(0, 0.5^2); chemists' ERI (ij|kl) = sum_{r < 2n} L_r[i,j] L_r[k,l] over symmetric factors L_r
    with entries N(0, 0.1^2) (8-fold symmetry); returned in the physicists' order of the MPO
    builders, vint[i,j,k,l] = (ik|jl)."""
    rng = np.random.default_rng(seed)

    def sym(scale):
        a = rng.normal(0.0, scale, size=(n, n))
        return np.triu(a) + np.triu(a, 1).T

    tkin = sym(0.5)
    L = np.stack([sym(0.1) for _ in range(2 * n)])
    eri = np.einsum("rij,rkl->ijkl", L, L)
    vint = np.ascontiguousarray(eri.transpose(0, 2, 1, 3))
    return tkin, vint


def complex_gauge(ch: cs.Chain, seed: int, bond_phases: bool = True, entry_phases: bool = False) -> cs.Chain:
    """complex128 copy of a chain (MPO or MPS). bond_phases: random phases on the virtual bonds,
    W_i[..., k] e^{i t_k} and W_{i+1}[k, ...] e^{-i t_k}, which leave the operator (or state)
    unchanged; entry_phases: a random phase on every entry (a different, genuinely complex state)."""
    rng = np.random.default_rng(seed)
    ts = []
    for t in ch.tensors:
        z = cs.BlockSparse(t.dim_logical, t.axis_dir, t.qnums_logical, dtype=cs.CT_DOUBLE_COMPLEX)
        for idx, b in t.blocks.items():
            z.blocks[idx] = b.astype(np.complex128)
            if entry_phases:
                z.blocks[idx] = z.blocks[idx] * np.exp(1j * rng.uniform(0.0, 2 * np.pi, size=b.shape))
        ts.append(z)
    if bond_phases:
        last = ts[0].ndim - 1
        for i in range(len(ts) - 1):
            ph = np.exp(1j * rng.uniform(0.0, 2 * np.pi, size=ts[i].dim_logical[last]))
            for t, ax, conj in ((ts[i], last, False), (ts[i + 1], 0, True)):
                for idx in list(t.blocks):
                    sel = np.nonzero(t.qnums_logical[ax] == t.qnums_blocks[ax][idx[ax]])[0]
                    shape = [1] * t.ndim
                    shape[ax] = len(sel)
                    f = np.conj(ph[sel]) if conj else ph[sel]
                    t.blocks[idx] = t.blocks[idx] * f.reshape(shape)
    return cs.Chain(ts, ch.qsite, ch.d)
