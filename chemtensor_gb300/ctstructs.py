"""ctypes mirror of chemtensor's C data structures and numpy conversions.

The C layouts follow include/ct_structs.h, which mirrors the reference's
struct dense_tensor (include/tensor/dense_tensor.h:17-23), struct
block_sparse_tensor (include/tensor/block_sparse_tensor.h:17-27), struct mps
(include/state/mps.h:14-20) and struct mpo (include/operator/mpo.h:34-40).

Every C-side array is allocated with libc ``aligned_alloc(16, ...)`` and
released with ``free``, which is the reference's ct_malloc / ct_free contract
(include/aligned_memory.h:17-54). That contract matters because
``dmrg_twosite`` frees the caller's MPS site tensors and allocates the
replacements itself.

On the Python side a block-sparse tensor is a :class:`BlockSparse`: logical
dimensions, axis directions, logical quantum numbers and a dict of dense
numpy blocks keyed by the block multi-index.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

ct_long = C.c_int64
qnumber = C.c_int32

CT_SINGLE_REAL, CT_DOUBLE_REAL, CT_SINGLE_COMPLEX, CT_DOUBLE_COMPLEX = 0, 1, 2, 3
TENSOR_AXIS_IN, TENSOR_AXIS_OUT = -1, 1


class DenseTensor(C.Structure):
    _fields_ = [
        ("data", C.c_void_p),
        ("dim", C.POINTER(ct_long)),
        ("dtype", C.c_int),
        ("ndim", C.c_int),
    ]


class BlockSparseTensor(C.Structure):
    _fields_ = [
        ("blocks", C.POINTER(C.POINTER(DenseTensor))),
        ("dim_blocks", C.POINTER(ct_long)),
        ("dim_logical", C.POINTER(ct_long)),
        ("axis_dir", C.POINTER(C.c_int)),
        ("qnums_blocks", C.POINTER(C.POINTER(qnumber))),
        ("qnums_logical", C.POINTER(C.POINTER(qnumber))),
        ("dtype", C.c_int),
        ("ndim", C.c_int),
    ]


class MPS(C.Structure):
    _fields_ = [
        ("a", C.POINTER(BlockSparseTensor)),
        ("qsite", C.POINTER(qnumber)),
        ("d", ct_long),
        ("nsites", C.c_int),
    ]


class MPO(C.Structure):
    _fields_ = [
        ("a", C.POINTER(BlockSparseTensor)),
        ("qsite", C.POINTER(qnumber)),
        ("d", ct_long),
        ("nsites", C.c_int),
    ]


_libc = C.CDLL("libc.so.6")
_libc.aligned_alloc.restype = C.c_void_p
_libc.aligned_alloc.argtypes = [C.c_size_t, C.c_size_t]
_libc.free.argtypes = [C.c_void_p]
_libc.free.restype = None


def _ct_malloc(nbytes: int) -> int:
    """aligned_alloc(16, nbytes rounded up to 16), as the reference's ct_malloc."""
    n = max(16, (int(nbytes) + 15) & ~15)
    p = _libc.aligned_alloc(16, n)
    if not p:
        raise MemoryError(f"aligned_alloc({n}) failed")
    C.memset(p, 0, n)
    return p


def _ct_free(p) -> None:
    if p:
        _libc.free(C.cast(p, C.c_void_p))


def _np_to_c(arr: np.ndarray, ctype):
    arr = np.ascontiguousarray(arr)
    p = _ct_malloc(arr.nbytes)
    C.memmove(p, arr.ctypes.data, arr.nbytes)
    return C.cast(p, C.POINTER(ctype))


# ---------------------------------------------------------------------------
# block structure rule (reference: allocate_block_sparse_tensor,
# src/tensor/block_sparse_tensor.c:37-151)
# ---------------------------------------------------------------------------

def block_structure(dims, axis_dir, qnums_logical):
    """Return (qnums_blocks, block_dims, allowed) for logical quantum numbers.

    ``qnums_blocks[i]`` are the sorted unique quantum numbers of axis i,
    ``block_dims[i][j]`` their multiplicities, and ``allowed`` the list of
    block multi-indices (row-major order) whose signed quantum numbers sum to
    zero. Integer arithmetic only, so the structure is exact.
    """
    qb, bd = [], []
    for i, q in enumerate(qnums_logical):
        q = np.asarray(q, dtype=np.int32)
        assert len(q) == dims[i] and dims[i] > 0
        u, c = np.unique(q, return_counts=True)
        qb.append(u.astype(np.int32))
        bd.append(c.astype(np.int64))
    allowed = []
    for idx in np.ndindex(*[len(u) for u in qb]):
        s = 0
        for i, j in enumerate(idx):
            s += int(axis_dir[i]) * int(qb[i][j])
        if s == 0:
            allowed.append(tuple(int(j) for j in idx))
    return qb, bd, allowed


@dataclass
class BlockSparse:
    """Host-side block-sparse tensor: dense numpy blocks keyed by block index."""

    dim_logical: tuple
    axis_dir: tuple
    qnums_logical: list
    blocks: dict = field(default_factory=dict)
    dtype: int = CT_DOUBLE_REAL

    def __post_init__(self):
        self.dim_logical = tuple(int(x) for x in self.dim_logical)
        self.axis_dir = tuple(int(x) for x in self.axis_dir)
        self.qnums_logical = [np.asarray(q, dtype=np.int32) for q in self.qnums_logical]
        self.qnums_blocks, self.block_dims, self.allowed = block_structure(
            self.dim_logical, self.axis_dir, self.qnums_logical)

    @property
    def ndim(self) -> int:
        return len(self.dim_logical)

    def npdtype(self):
        return {CT_SINGLE_REAL: np.float32, CT_DOUBLE_REAL: np.float64,
                CT_SINGLE_COMPLEX: np.complex64, CT_DOUBLE_COMPLEX: np.complex128}[self.dtype]

    def block_shape(self, idx):
        return tuple(int(self.block_dims[i][j]) for i, j in enumerate(idx))

    def zeros_like_structure(self):
        for idx in self.allowed:
            self.blocks[idx] = np.zeros(self.block_shape(idx), dtype=self.npdtype())
        return self

    def num_elements_blocks(self) -> int:
        return int(sum(np.prod(self.block_shape(idx)) for idx in self.allowed))

    def serialize(self) -> np.ndarray:
        """Concatenate blocks in block-index order (reference:
        block_sparse_tensor_serialize_entries, block_sparse_tensor.c:3131)."""
        if not self.allowed:
            return np.zeros(0, dtype=self.npdtype())
        return np.concatenate([self.blocks[idx].ravel() for idx in self.allowed])

    def to_dense(self) -> np.ndarray:
        out = np.zeros(self.dim_logical, dtype=self.npdtype())
        maps = [[np.nonzero(self.qnums_logical[i] == q)[0] for q in self.qnums_blocks[i]]
                for i in range(self.ndim)]
        for idx, b in self.blocks.items():
            out[np.ix_(*[maps[i][j] for i, j in enumerate(idx)])] = b
        return out


# ---------------------------------------------------------------------------
# C <-> Python
# ---------------------------------------------------------------------------

def read_bst(t: BlockSparseTensor) -> BlockSparse:
    nd = t.ndim
    dims = [t.dim_logical[i] for i in range(nd)]
    dirs = [t.axis_dir[i] for i in range(nd)]
    qn = [np.ctypeslib.as_array(t.qnums_logical[i], shape=(dims[i],)).copy() for i in range(nd)]
    bs = BlockSparse(dims, dirs, qn, dtype=t.dtype)
    dimb = [t.dim_blocks[i] for i in range(nd)]
    for i in range(nd):
        qbc = np.ctypeslib.as_array(t.qnums_blocks[i], shape=(dimb[i],))
        if not np.array_equal(qbc, bs.qnums_blocks[i]):
            raise ValueError("C tensor block quantum numbers are not the sorted unique logical ones")
    npdt = bs.npdtype()
    for idx in bs.allowed:
        k = int(np.ravel_multi_index(idx, dimb)) if nd > 0 else 0
        if not t.blocks[k]:
            raise ValueError(f"missing block {idx}")
        b = t.blocks[k].contents
        shape = tuple(b.dim[i] for i in range(b.ndim))
        if shape != bs.block_shape(idx):
            raise ValueError(f"block {idx} has shape {shape}, expected {bs.block_shape(idx)}")
        n = int(np.prod(shape))
        buf = (C.c_char * (n * np.dtype(npdt).itemsize)).from_address(b.data)
        bs.blocks[idx] = np.frombuffer(buf, dtype=npdt).reshape(shape).copy()
    return bs


def write_bst(bs: BlockSparse, t: BlockSparseTensor) -> None:
    """Fill the C struct ``t`` with freshly allocated copies of ``bs``."""
    nd = bs.ndim
    t.ndim = nd
    t.dtype = bs.dtype
    t.dim_logical = _np_to_c(np.array(bs.dim_logical, dtype=np.int64), ct_long)
    t.dim_blocks = _np_to_c(np.array([len(q) for q in bs.qnums_blocks], dtype=np.int64), ct_long)
    t.axis_dir = _np_to_c(np.array(bs.axis_dir, dtype=np.int32), C.c_int)
    ql = C.cast(_ct_malloc(nd * C.sizeof(C.c_void_p)), C.POINTER(C.POINTER(qnumber)))
    qbp = C.cast(_ct_malloc(nd * C.sizeof(C.c_void_p)), C.POINTER(C.POINTER(qnumber)))
    for i in range(nd):
        ql[i] = _np_to_c(bs.qnums_logical[i].astype(np.int32), qnumber)
        qbp[i] = _np_to_c(bs.qnums_blocks[i].astype(np.int32), qnumber)
    t.qnums_logical = ql
    t.qnums_blocks = qbp
    dimb = [len(q) for q in bs.qnums_blocks]
    nblocks = int(np.prod(dimb))
    blocks = C.cast(_ct_malloc(nblocks * C.sizeof(C.c_void_p)), C.POINTER(C.POINTER(DenseTensor)))
    npdt = bs.npdtype()
    for idx in bs.allowed:
        k = int(np.ravel_multi_index(idx, dimb))
        shape = bs.block_shape(idx)
        arr = bs.blocks.get(idx)
        if arr is None:
            arr = np.zeros(shape, dtype=npdt)
        arr = np.ascontiguousarray(arr, dtype=npdt)
        assert arr.shape == shape
        d = C.cast(_ct_malloc(C.sizeof(DenseTensor)), C.POINTER(DenseTensor))
        d.contents.ndim = nd
        d.contents.dtype = bs.dtype
        d.contents.dim = _np_to_c(np.array(shape, dtype=np.int64), ct_long)
        d.contents.data = C.cast(_np_to_c(arr, C.c_char), C.c_void_p)
        blocks[k] = d
    t.blocks = blocks


def free_bst(t: BlockSparseTensor) -> None:
    """Release a C tensor as the reference's delete_block_sparse_tensor does."""
    nd = t.ndim
    if t.blocks:
        nblocks = 1
        for i in range(nd):
            nblocks *= t.dim_blocks[i]
        for k in range(nblocks):
            if t.blocks[k]:
                b = t.blocks[k].contents
                _ct_free(b.data)
                _ct_free(b.dim)
                _ct_free(t.blocks[k])
        _ct_free(t.blocks)
    for i in range(nd):
        if t.qnums_blocks:
            _ct_free(t.qnums_blocks[i])
        if t.qnums_logical:
            _ct_free(t.qnums_logical[i])
    _ct_free(t.qnums_blocks)
    _ct_free(t.qnums_logical)
    _ct_free(t.axis_dir)
    _ct_free(t.dim_blocks)
    _ct_free(t.dim_logical)
    t.blocks = None
    t.ndim = 0


@dataclass
class Chain:
    """Host-side MPS or MPO: a list of BlockSparse site tensors."""

    tensors: list
    qsite: np.ndarray
    d: int

    @property
    def nsites(self) -> int:
        return len(self.tensors)

    def bond_dims(self):
        return [t.dim_logical[0] for t in self.tensors] + [self.tensors[-1].dim_logical[-1]]


def _read_chain(c) -> Chain:
    ts = [read_bst(c.a[i]) for i in range(c.nsites)]
    qsite = np.ctypeslib.as_array(c.qsite, shape=(c.d,)).copy()
    return Chain(ts, qsite, int(c.d))


def _write_chain(ch: Chain, c) -> None:
    c.nsites = ch.nsites
    c.d = ch.d
    c.qsite = _np_to_c(np.asarray(ch.qsite, dtype=np.int32), qnumber)
    arr = C.cast(_ct_malloc(ch.nsites * C.sizeof(BlockSparseTensor)), C.POINTER(BlockSparseTensor))
    for i, t in enumerate(ch.tensors):
        write_bst(t, arr[i])
    c.a = arr


def _free_chain(c) -> None:
    if c.a:
        for i in range(c.nsites):
            free_bst(c.a[i])
        _ct_free(c.a)
    _ct_free(c.qsite)
    c.a = None
    c.qsite = None
    c.nsites = 0


def read_mps(c: MPS) -> Chain:
    return _read_chain(c)


def read_mpo(c: MPO) -> Chain:
    return _read_chain(c)


def make_c_mps(ch: Chain) -> MPS:
    c = MPS()
    _write_chain(ch, c)
    return c


def make_c_mpo(ch: Chain) -> MPO:
    c = MPO()
    _write_chain(ch, c)
    return c


def free_mps(c: MPS) -> None:
    _free_chain(c)


def free_mpo(c: MPO) -> None:
    _free_chain(c)


# ---------------------------------------------------------------------------
# flat array form (golden fixtures, .npz)
# ---------------------------------------------------------------------------

def bst_to_arrays(prefix: str, t: BlockSparse) -> dict:
    cplx = t.dtype == CT_DOUBLE_COMPLEX
    out = {f"{prefix}_dim": np.array(t.dim_logical, dtype=np.int64),
           f"{prefix}_dir": np.array(t.axis_dir, dtype=np.int32),
           f"{prefix}_data": t.serialize().astype(np.complex128 if cplx else np.float64)}
    if cplx:
        out[f"{prefix}_dtype"] = np.array(CT_DOUBLE_COMPLEX)
    for i, q in enumerate(t.qnums_logical):
        out[f"{prefix}_q{i}"] = np.asarray(q, dtype=np.int32)
    return out


def bst_from_arrays(prefix: str, arr) -> BlockSparse:
    dim = [int(x) for x in arr[f"{prefix}_dim"]]
    dirs = [int(x) for x in arr[f"{prefix}_dir"]]
    qn = [np.asarray(arr[f"{prefix}_q{i}"], dtype=np.int32) for i in range(len(dim))]
    cplx = f"{prefix}_dtype" in arr and int(arr[f"{prefix}_dtype"]) == CT_DOUBLE_COMPLEX
    t = BlockSparse(dim, dirs, qn, dtype=CT_DOUBLE_COMPLEX if cplx else CT_DOUBLE_REAL)
    data = np.asarray(arr[f"{prefix}_data"], dtype=np.complex128 if cplx else np.float64)
    off = 0
    for idx in t.allowed:
        shp = t.block_shape(idx)
        n = int(np.prod(shp))
        t.blocks[idx] = data[off:off + n].reshape(shp).copy()
        off += n
    if off != len(data):
        raise ValueError(f"{prefix}: {len(data)} entries for {off} block entries")
    return t


def chain_to_arrays(prefix: str, ch: Chain) -> dict:
    out = {f"{prefix}_nsites": np.array(ch.nsites), f"{prefix}_d": np.array(ch.d),
           f"{prefix}_qsite": np.asarray(ch.qsite, dtype=np.int32)}
    for i, t in enumerate(ch.tensors):
        out.update(bst_to_arrays(f"{prefix}{i}", t))
    return out


def chain_from_arrays(prefix: str, arr) -> Chain:
    n = int(arr[f"{prefix}_nsites"])
    ts = [bst_from_arrays(f"{prefix}{i}", arr) for i in range(n)]
    return Chain(ts, np.asarray(arr[f"{prefix}_qsite"], dtype=np.int32), int(arr[f"{prefix}_d"]))
