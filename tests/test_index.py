"""Particle-ID -> index tables (hbtu_index_*, hbtplus_gb300.index), the ID
re-resolve of the unbinding step's callers (IndexTable_t, src/hash.h:47-112).

CPU: the C restatement (oracle) reproduces the reference's own
MappedIndexTable_t and FlatIndexTable_t answers stored in
tests/golden/index_*.npz (made by tests/golden/make_golden.py from the
reference build), for single lookups (GetIndex) and the batch form on sorted
queries (GetIndices).
GPU: the GPU tables give the same answers bit for bit, on the fixtures, on
random tables against the oracle (hits, misses, negative and out-of-range
keys, duplicate keys with the documented rule), through device-resident
tensors, and at 3e7 keys (a bijection: every ID maps back to its position).
"""
import os
import sys

import numpy as np
import pytest

from helpers import GOLDEN

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="module")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.mark.parametrize("name,flat", [("index_mapped", False), ("index_flat", True)])
def test_oracle_matches_reference_fixture(oracle, name, flat):
    g = golden(name)
    null = int(g["null_index"])
    out = oracle.index_lookup(g["keys"], g["values"], g["queries"], flat=flat, null_index=null)
    assert np.array_equal(out, g["ref_out"])
    out = oracle.index_lookup(g["keys"], g["values"], g["sorted_queries"], flat=flat,
                              null_index=null)
    assert np.array_equal(out, g["ref_out_sorted"])
    assert 0 < np.sum(out != null) < len(out)  # hits and misses


def test_oracle_duplicate_rule(oracle):
    keys = np.array([5, 3, 5, 9, 3], np.int64)
    vals = np.array([10, 11, 12, 13, 14], np.int64)
    q = np.array([3, 5, 9, 4, -1], np.int64)
    assert list(oracle.index_lookup(keys, vals, q, flat=False)) == [11, 10, 13, -1, -1]
    assert list(oracle.index_lookup(keys, vals, q, flat=True)) == [14, 12, 13, -1, -1]


# ------------------------------------------------------------------- GPU
def tables(flat):
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.index import FlatIndexTable, MappedIndexTable
    from hbtplus_gb300.unbind import Unbinder
    ub = Unbinder(S.default_params())
    return ub, (FlatIndexTable if flat else MappedIndexTable)(ub)


@pytest.mark.gpu
@pytest.mark.parametrize("name,flat", [("index_mapped", False), ("index_flat", True)])
def test_gpu_matches_reference_fixture(name, flat):
    g = golden(name)
    ub, t = tables(flat)
    t.Fill(g["keys"], g["values"], null_index=int(g["null_index"]))
    assert np.array_equal(t.GetIndices(g["queries"]), g["ref_out"])
    assert np.array_equal(t.GetIndices(g["sorted_queries"]), g["ref_out_sorted"])
    assert t.GetKeyMinMax() == (int(g["keys"].min()), int(g["keys"].max()))
    t.close()
    ub.close()


@pytest.mark.gpu
@pytest.mark.parametrize("flat", [False, True])
def test_gpu_matches_oracle_random(oracle, flat):
    rng = np.random.default_rng(3 + flat)
    ub, t = tables(flat)
    for trial in range(12):
        n = int(rng.integers(0, 60000))
        span = int(rng.integers(max(n, 1), 3 * max(n, 1) + 50))
        base = int(rng.integers(-1000, 10**9)) if not flat else int(rng.integers(0, 10**6))
        keys = rng.integers(0, span, n).astype(np.int64) + base  # duplicates included
        vals = rng.integers(-10**12, 10**12, n).astype(np.int64)
        q = np.concatenate([keys[: n // 3], rng.integers(base - 100, base + span + 100, 20000),
                            np.array([-1, -(2**62), 2**62])]).astype(np.int64)
        null = int(rng.integers(-5, 5))
        t.Fill(keys, vals, null_index=null)
        expect = oracle.index_lookup(keys, vals, q, flat=flat, null_index=null)
        assert np.array_equal(t.GetIndices(q), expect), (trial, n)
    t.close()
    ub.close()


@pytest.mark.gpu
def test_gpu_empty_and_limits():
    from hbtplus_gb300 import _lib
    for flat in (False, True):
        ub, t = tables(flat)
        t.Fill(np.zeros(0, np.int64), np.zeros(0, np.int64), null_index=-3)
        assert list(t.GetIndices(np.array([0, 5, -1], np.int64))) == [-3, -3, -3]
        t.close()
        ub.close()
    ub, t = tables(True)  # a flat table over a key span above 2^32 is refused
    with pytest.raises(_lib.HBTUError):
        t.Fill(np.array([0, 2**33], np.int64), np.array([0, 1], np.int64))
    t.close()
    ub.close()


@pytest.mark.gpu
@pytest.mark.parametrize("flat", [False, True])
def test_gpu_device_resident_30m(flat):
    """3e7 IDs (a 200 Mpc/h snapshot's particle count): sparse shuffled IDs
    for the mapped table, a dense permuted range for the flat one.  Every ID
    maps back to its position; absent IDs give the null index."""
    torch = pytest.importorskip("torch")
    n = 30_000_000
    g = torch.Generator(device="cuda").manual_seed(11)
    if flat:
        ids = torch.randperm(n, device="cuda", generator=g).to(torch.int64) + 1000
    else:
        ids = torch.randperm(4 * n, device="cuda", generator=g)[:n].to(torch.int64) * 7 + 3
    pos = torch.arange(n, device="cuda", dtype=torch.int64)
    ub, t = tables(flat)
    ub.set_stream(torch.cuda.current_stream().cuda_stream)
    t.fill_device(ids, pos, null_index=-1)
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    perm = torch.randperm(n, device="cuda", generator=g)
    t.lookup_device(ids[perm], out)
    torch.cuda.synchronize()
    assert torch.equal(out, perm)
    miss = (ids[:1000] + (1 if not flat else n)).contiguous()  # ids*7+3+1 never occur
    t.lookup_device(miss, out[:1000])
    torch.cuda.synchronize()
    assert bool((out[:1000] == -1).all())
    t.close()
    ub.close()
