"""Particle-ID -> index tables on the GPU, mirroring the reference's
IndexTable_t (src/hash.h:47-112): MappedIndexTable_t (the reference's sorted
pairs and binary search; a hash table here, same answers) and
FlatIndexTable_t (dense array over the key range).

    with Unbinder(params) as ub:
        table = MappedIndexTable(ub)              # or FlatIndexTable(ub)
        table.Fill(ids, np.arange(len(ids)), null_index=-1)
        idx = table.GetIndices(query_ids)          # GetIndex of every query
        kmin, kmax = table.GetKeyMinMax()

Host numpy arrays go through host staging; CUDA torch tensors stay on the
device (fill_device / lookup_device).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class _IndexTable:
    _flat = 0

    def __init__(self, unbinder):
        self.ub = unbinder
        self.lib = unbinder.lib
        self.t = C.c_void_p()
        _lib.check(self.lib.hbtu_index_create(unbinder.handle, self._flat, C.byref(self.t)),
                   unbinder.handle)
        self.NullIndex = -1

    def close(self) -> None:
        if self.t:
            self.lib.hbtu_index_destroy(self.t)
            self.t = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- the reference's interface -----------------------------------------
    def Fill(self, keys, values=None, null_index: int = -1) -> None:
        """IndexTable_t::Fill: pairs (keys[i], values[i]); values default to
        the positions 0..n-1 (a snapshot's particle index)."""
        k = np.ascontiguousarray(keys, np.int64)
        v = (np.arange(len(k), dtype=np.int64) if values is None
             else np.ascontiguousarray(values, np.int64))
        if len(v) != len(k):
            raise ValueError("keys and values differ in length")
        self.NullIndex = int(null_index)
        _lib.check(self.lib.hbtu_index_fill(self.t, k.ctypes.data if len(k) else None,
                                            v.ctypes.data if len(v) else None, len(k),
                                            int(null_index), _lib.HBTU_HOST), self.ub.handle)

    def GetIndex(self, key: int) -> int:
        return int(self.GetIndices(np.array([key], np.int64))[0])

    def GetIndices(self, keys) -> np.ndarray:
        q = np.ascontiguousarray(keys, np.int64)
        out = np.empty(max(len(q), 1), np.int64)
        _lib.check(self.lib.hbtu_index_lookup(self.t, q.ctypes.data if len(q) else None, len(q),
                                              out.ctypes.data, _lib.HBTU_HOST), self.ub.handle)
        return out[:len(q)]

    def GetKeyMinMax(self):
        lo, hi = C.c_int64(), C.c_int64()
        _lib.check(self.lib.hbtu_index_key_range(self.t, C.byref(lo), C.byref(hi)),
                   self.ub.handle)
        return lo.value, hi.value

    # -- device-resident forms (int64 CUDA tensors on the handle's device) --
    def fill_device(self, keys, values, null_index: int = -1) -> None:
        self.NullIndex = int(null_index)
        _lib.check(self.lib.hbtu_index_fill(self.t, keys.data_ptr(), values.data_ptr(),
                                            keys.numel(), int(null_index), _lib.HBTU_DEVICE),
                   self.ub.handle)

    def lookup_device(self, keys, out) -> None:
        _lib.check(self.lib.hbtu_index_lookup(self.t, keys.data_ptr(), keys.numel(),
                                              out.data_ptr(), _lib.HBTU_DEVICE), self.ub.handle)


class MappedIndexTable(_IndexTable):
    """MappedIndexTable_t (src/hash.tpp:18-55): the reference sorts the pairs
    and binary-searches them; here a GPU hash table with the same answers."""
    _flat = 0


class FlatIndexTable(_IndexTable):
    """FlatIndexTable_t (src/hash.tpp:59-109): dense array over the key range."""
    _flat = 1
