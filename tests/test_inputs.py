"""Host-side input builders against the reference (CPU only; no GPU calls)."""

import re
import os

import numpy as np
import pytest

from chemtensor_gb300 import ctstructs as cs, hamiltonians as hm
from conftest import ROOT, golden


def test_randn_sequences_bitwise(gpu):
    g = golden("rng_sequences.npz")
    for key in g.files:
        seed = int(key.split("_")[1])
        out = np.zeros(2000)
        gpu.ctgpu_randn_sequence(seed, 2000, out.ctypes.data)
        assert np.array_equal(out, g[key]), key


@pytest.mark.parametrize("tag", ["heis_L12_D8_s1", "hub_L8_D24_s3", "hub_L10_D16_s42"])
def test_random_mps_bitwise(gpu, tag):
    from chemtensor_gb300 import native
    g = golden("random_mps.npz")
    L, sector, D, seed = [int(x) for x in g[f"{tag}_params"]]
    ref = cs.chain_from_arrays(tag, g)
    c = native.random_mps(L, ref.d, ref.qsite, sector, D, seed)
    mine = cs.read_mps(c)
    cs.free_mps(c)
    for a, b in zip(mine.tensors, ref.tensors):
        assert a.dim_logical == b.dim_logical
        assert all(np.array_equal(x, y) for x, y in zip(a.qnums_logical, b.qnums_logical))
        assert np.array_equal(a.serialize(), b.serialize())


@pytest.mark.parametrize("tag", ["heis_L12_D8_s1", "hub_L8_D24_s3", "hub_L10_D16_s42"])
def test_oracle_random_mps_bitwise(oracle_port, tag):
    """The oracle's own seeded generator (used by the CPU baseline, which loads no GPU library)
    reproduces the reference's construct_random_mps bit for bit."""
    import ctypes as C
    g = golden("random_mps.npz")
    L, sector, D, seed = [int(x) for x in g[f"{tag}_params"]]
    ref = cs.chain_from_arrays(tag, g)
    q = np.ascontiguousarray(ref.qsite, dtype=np.int32)
    c = cs.MPS()
    assert oracle_port.oracle_construct_random_mps(L, ref.d, q.ctypes.data, sector, D, seed, C.byref(c)) == 0
    mine = cs.read_mps(c)
    cs.free_mps(c)
    for a, b in zip(mine.tensors, ref.tensors):
        assert a.dim_logical == b.dim_logical
        assert all(np.array_equal(x, y) for x, y in zip(a.qnums_logical, b.qnums_logical))
        assert np.array_equal(a.serialize(), b.serialize())


def test_heisenberg_mpo_equals_reference_operator():
    g = golden("mpo_reference.npz")
    a = hm.mpo_to_matrix(cs.chain_from_arrays("heis6", g))
    b = hm.mpo_to_matrix(hm.heisenberg_xxz_1d(6, 1.0, 0.8, 0.3))
    assert np.abs(a - b).max() < 1e-14


def test_hubbard_mpo_equals_reference_operator():
    g = golden("mpo_reference.npz")
    a = hm.mpo_to_matrix(cs.chain_from_arrays("hub4", g))
    b = hm.mpo_to_matrix(hm.fermi_hubbard_1d(4, 1.0, 4.0, 0.3))
    assert np.abs(a - b).max() < 1e-14


def test_struct_round_trip():
    ch = hm.fermi_hubbard_1d(5, 1.0, 2.0, 0.1)
    c = cs.make_c_mpo(ch)
    back = cs.read_mpo(c)
    cs.free_mpo(c)
    for x, y in zip(ch.tensors, back.tensors):
        assert np.array_equal(x.serialize(), y.serialize())


def test_library_exports_every_declared_symbol(gpu):
    text = open(os.path.join(ROOT, "include", "ctgpu.h")).read()
    names = set(re.findall(r"^\s*(?:int|void|const char\*)\s+\**(\w+)\s*\(", text, flags=re.M))
    assert "dmrg_twosite" in names and len(names) >= 10
    for n in names:
        assert hasattr(gpu, n), n


def test_oracle_exports(oracle_port):
    text = open(os.path.join(ROOT, "oracle", "ct_oracle.h")).read()
    names = set(re.findall(r"^\s*(?:int|void|double|ct_long)\s+\**(\w+)\s*\(", text, flags=re.M))
    assert len(names) >= 10
    for n in names:
        assert hasattr(oracle_port, n), n
